// Several right-hand sides solved together (the combined form): the block
// operator apply reads each element's qdata once for all R vectors, and a block
// PCG runs R independent CGSolver recurrences (linalg/solvers.cpp:869-1050,
// one set of scalars per right-hand side) on vectors stored interleaved,
// v[i*R + r]. A mixed-precision block solve wraps FP32 block PCG in FP64 defect
// correction with FP64 true residuals, per right-hand side.
#include "gbpa_csr.cuh"
#include "gbpa_operator.cuh"
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace gbpa
{
int launch_diffusion_block_f64(gbpa_ctx *ctx, int ne, int nrhs, int symm, int D, int Q,
                               const double *B, const double *G, const double *qd, const double *x,
                               const int *gather_map, const unsigned char *ess_mask, double *y,
                               const int *skip);
int launch_diffusion_block_f32(gbpa_ctx *ctx, int ne, int nrhs, int symm, int D, int Q,
                               const float *B, const float *G, const float *qd, const float *x,
                               const int *gather_map, const unsigned char *ess_mask, float *y,
                               const int *skip);

constexpr int BK_BLOCK = 512;   // a multiple of every supported R (1, 2, 4, 8)
constexpr int BK_MAXR = 8;

struct BlockState
{
   double nom[BK_MAXR], nom0[BK_MAXR], den[BK_MAXR], betanom[BK_MAXR];
   double alpha[BK_MAXR], beta[BK_MAXR], r0[BK_MAXR];
   int iter[BK_MAXR], done[BK_MAXR], converged[BK_MAXR], final_iter[BK_MAXR];
   int status, all_done, nrhs, max_it;
   double rel2, abs2;
   unsigned int counter[4];
};

// Sums of a per-thread value grouped by right-hand side r = threadIdx.x % R
// (the grid-stride step is a multiple of R, so each thread keeps one r).
// block_sum_rhs: block sums of s grouped by r, in a fixed order; on return
// out[r] (shared) holds them for every thread.
__device__ void block_sum_rhs(double s, int R, double *out)
{
   __shared__ double ws[32][BK_MAXR];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   for (int o = 16; o >= R; o >>= 1) { s += __shfl_down_sync(0xffffffffu, s, o); }
   if (lane < R) { ws[wid][lane] = s; }
   __syncthreads();
   if (threadIdx.x < R)
   {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { t += ws[w][threadIdx.x]; }
      out[threadIdx.x] = t;
   }
   __syncthreads();
}

// Publishes the block's R partials; returns true in the last block, where
// tot[r] (shared) holds the grid totals. The last block reads the partials
// with all its threads (thread t takes blocks t / R, t / R + blockDim.x / R,
// ... of right-hand side t % R) and reduces them with the same fixed-order
// tree, so the totals are deterministic for a given grid.
__device__ bool publish_rhs(int R, double *partials, unsigned int *counter, double *tot)
{
   __shared__ bool last;
   if (threadIdx.x < R)
   {
      partials[blockIdx.x * R + threadIdx.x] = tot[threadIdx.x];
      __threadfence();
   }
   __syncthreads();
   if (threadIdx.x == 0) { last = atomicInc(counter, gridDim.x - 1) == gridDim.x - 1; }
   __syncthreads();
   if (!last) { return false; }
   __threadfence();
   const int q = threadIdx.x % R, G = blockDim.x / R;
   double t = 0.0;
   for (int b = threadIdx.x / R; b < (int)gridDim.x; b += G) { t += __ldcg(partials + b * R + q); }
   block_sum_rhs(t, R, tot);
   return true;
}

__device__ bool finish_rhs(double s, int R, double *partials, unsigned int *counter, double *tot)
{
   block_sum_rhs(s, R, tot);
   return publish_rhs(R, partials, counter, tot);
}

// Block sums of a thread's R values s[r], in a fixed order; on return out[r]
// (shared) holds them for every thread.
template <int R>
__device__ void block_sum_vec(double (&s)[R], double *out)
{
   __shared__ double ws[32][R];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
   for (int r = 0; r < R; ++r)
   {
      for (int o = 16; o > 0; o >>= 1) { s[r] += __shfl_down_sync(0xffffffffu, s[r], o); }
   }
   if (lane == 0)
   {
#pragma unroll
      for (int r = 0; r < R; ++r) { ws[wid][r] = s[r]; }
   }
   __syncthreads();
   if (threadIdx.x < R)
   {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { t += ws[w][threadIdx.x]; }
      out[threadIdx.x] = t;
   }
   __syncthreads();
}

template <typename T>
__global__ void blk_init_kernel(int64_t n, int R, const T *__restrict__ b, T *__restrict__ x,
                                T *__restrict__ r, T *__restrict__ z, T *__restrict__ d,
                                const T *__restrict__ dinv, double *partials, BlockState *st)
{
   __shared__ double tot[BK_MAXR];
   double s = 0.0;
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      const T rk = b[k];
      x[k] = T(0);
      r[k] = rk;
      const T zk = dinv[k >> (__ffs(R) - 1)] * rk;
      z[k] = zk;
      d[k] = zk;
      s += (double)zk * (double)rk;
   }
   if (finish_rhs(s, R, partials, &st->counter[0], tot) && threadIdx.x == 0)
   {
      int active = 0;
      for (int q = 0; q < R; ++q)
      {
         const double nom = tot[q];
         st->nom[q] = st->nom0[q] = st->betanom[q] = nom;
         st->iter[q] = 1; st->converged[q] = 0; st->final_iter[q] = 0; st->done[q] = 0;
         if (!isfinite(nom)) { st->status = GBPA_ERR_NOT_FINITE; st->done[q] = 1; }
         else if (nom < 0.0) { st->done[q] = 1; }
         else
         {
            st->r0[q] = fmax(nom * st->rel2, st->abs2);
            if (nom <= st->r0[q]) { st->converged[q] = 1; st->done[q] = 1; }
         }
         active += !st->done[q];
      }
      st->all_done = active == 0;
   }
}

// z = CSR scatter of the block E-vector (z[ess] = d[ess]) and den_r = (d_r, z_r),
// one thread per dof for all R right-hand sides (vector loads of the R
// interleaved values; z and d are internal, so aligned to R * sizeof(T)).
template <typename T, int R>
__global__ void blk_scatter_den_kernel(int ndofs, const int *__restrict__ offsets,
                                       const int *__restrict__ indices, const T *__restrict__ yE,
                                       T *__restrict__ z, const T *__restrict__ d,
                                       const unsigned char *__restrict__ mask, double *partials,
                                       BlockState *st, int first)
{
   if (st->all_done) { return; }
   using V = RhsVec<T, R>;
   __shared__ double tot[BK_MAXR];
   double s[R];
#pragma unroll
   for (int r = 0; r < R; ++r) { s[r] = 0.0; }
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndofs; i += gridDim.x * blockDim.x)
   {
      const V dv = reinterpret_cast<const V *>(d)[i];
      V v;
      if (mask && mask[i]) { v = dv; }
      else { csr_row_sum_rhs<T, R>(offsets, indices, yE, i, v.v); }
      reinterpret_cast<V *>(z)[i] = v;
#pragma unroll
      for (int r = 0; r < R; ++r) { s[r] += (double)dv.v[r] * (double)v.v[r]; }
   }
   block_sum_vec<R>(s, tot);
   if (publish_rhs(R, partials, &st->counter[1], tot) && threadIdx.x == 0)
   {
      int active = 0;
      for (int q = 0; q < R; ++q)
      {
         if (!st->done[q])
         {
            const double den = tot[q];
            st->den[q] = den;
            if (!isfinite(den)) { st->status = GBPA_ERR_NOT_FINITE; st->done[q] = 1; st->final_iter[q] = st->iter[q]; }
            else if (den == 0.0) { st->done[q] = 1; st->final_iter[q] = st->iter[q]; }
            else
            {
               if (!first) { st->nom[q] = st->betanom[q]; }
               st->alpha[q] = st->nom[q] / den;
            }
         }
         active += !st->done[q];
      }
      st->all_done = active == 0;
   }
}

template <typename T>
__global__ void blk_update_kernel(int64_t n, int R, T *__restrict__ x, T *__restrict__ r,
                                  T *__restrict__ z, const T *__restrict__ d,
                                  const T *__restrict__ dinv, double *partials, BlockState *st)
{
   if (st->all_done) { return; }
   __shared__ double tot[BK_MAXR];
   const int q = threadIdx.x % R;
   const T alpha = st->done[q] ? T(0) : (T)st->alpha[q];
   double s = 0.0;
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      x[k] += alpha * d[k];
      const T rk = r[k] - alpha * z[k];
      r[k] = rk;
      const T zk = dinv[k >> (__ffs(R) - 1)] * rk;
      z[k] = zk;
      s += (double)rk * (double)zk;
   }
   if (finish_rhs(s, R, partials, &st->counter[2], tot) && threadIdx.x == 0)
   {
      int active = 0;
      for (int c = 0; c < R; ++c)
      {
         if (!st->done[c])
         {
            const double bn = tot[c];
            st->betanom[c] = bn;
            if (!isfinite(bn)) { st->status = GBPA_ERR_NOT_FINITE; st->done[c] = 1; st->final_iter[c] = st->iter[c]; }
            else if (bn < 0.0) { st->done[c] = 1; st->final_iter[c] = st->iter[c]; }
            else if (bn <= st->r0[c]) { st->converged[c] = 1; st->done[c] = 1; st->final_iter[c] = st->iter[c]; }
            else if (++st->iter[c] > st->max_it) { st->done[c] = 1; st->final_iter[c] = st->max_it; }
            else { st->beta[c] = bn / st->nom[c]; }
         }
         active += !st->done[c];
      }
      st->all_done = active == 0;
   }
}

template <typename T>
__global__ void blk_direction_kernel(int64_t n, int R, const T *__restrict__ z, T *__restrict__ d,
                                     const BlockState *st)
{
   if (st->all_done) { return; }
   const int q = threadIdx.x % R;
   if (st->done[q]) { return; }
   const T beta = (T)st->beta[q];
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      d[k] = z[k] + beta * d[k];
   }
}

template <typename T>
__global__ void blk_scatter_kernel(int ndofs, int R, const int *__restrict__ offsets,
                                   const int *__restrict__ indices, const T *__restrict__ yE,
                                   T *__restrict__ y, const unsigned char *__restrict__ mask,
                                   const T *__restrict__ xc)
{
   const int64_t n = (int64_t)ndofs * R;
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      const int i = (int)(k >> (__ffs(R) - 1)), q = (int)(k & (R - 1));   // R is a power of two
      if (mask && mask[i]) { y[k] = xc[k]; continue; }
      y[k] = csr_row_sum<T>(offsets, indices, yE, i, false, R, q);
   }
}

// The same with one thread per dof for all R right-hand sides: the row's
// indices loaded once, R values per slot in one vector load (bit-identical
// sums); y and xc aligned to R * sizeof(T).
template <typename T, int R>
__global__ void blk_scatter_rhs_kernel(int ndofs, const int *__restrict__ offsets,
                                       const int *__restrict__ indices, const T *__restrict__ yE,
                                       T *__restrict__ y, const unsigned char *__restrict__ mask,
                                       const T *__restrict__ xc)
{
   using V = RhsVec<T, R>;
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndofs; i += gridDim.x * blockDim.x)
   {
      V v;
      if (mask && mask[i]) { v = reinterpret_cast<const V *>(xc)[i]; }
      else { csr_row_sum_rhs<T, R>(offsets, indices, yE, i, v.v); }
      reinterpret_cast<V *>(y)[i] = v;
   }
}

// per-right-hand-side dot products (a, b) -> out[R] (device)
template <typename T>
__global__ void blk_dot_kernel(int64_t n, int R, const T *__restrict__ a, const T *__restrict__ b,
                               double *partials, unsigned int *counter, double *out)
{
   __shared__ double tot[BK_MAXR];
   double s = 0.0;
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      s += (double)a[k] * (double)b[k];
   }
   if (finish_rhs(s, R, partials, counter, tot) && threadIdx.x < R) { out[threadIdx.x] = tot[threadIdx.x]; }
}

// Reliable update of the FP32 block PCG (residuals already replaced by the
// true ones, zero where converged): z = dinv r, betanom_r = (r_r, z_r),
// beta_r = betanom_r / nom_r, next segment level r0_r = rel2 * betanom_r
// (rel2 holds delta^2); converged right-hand sides stay done.
__global__ void blk_restart_kernel(int64_t n, int R, const float *__restrict__ r,
                                   float *__restrict__ z, const float *__restrict__ dinv,
                                   const int *__restrict__ conv, double *partials, BlockState *st)
{
   __shared__ double tot[BK_MAXR];
   double s = 0.0;
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      const float zk = dinv[k >> (__ffs(R) - 1)] * r[k];
      z[k] = zk;
      s += (double)r[k] * (double)zk;
   }
   if (finish_rhs(s, R, partials, &st->counter[3], tot) && threadIdx.x == 0)
   {
      int active = 0;
      for (int q = 0; q < R; ++q)
      {
         if (conv[q]) { st->done[q] = 1; continue; }
         const double bn = tot[q];
         st->betanom[q] = bn;
         st->converged[q] = 0;
         st->done[q] = 0;
         if (!isfinite(bn)) { st->status = GBPA_ERR_NOT_FINITE; st->done[q] = 1; st->final_iter[q] = st->iter[q]; }
         else if (bn <= 0.0) { st->done[q] = 1; st->final_iter[q] = st->iter[q]; }
         else
         {
            st->beta[q] = bn / st->nom[q];
            st->r0[q] = st->rel2 * bn;
         }
         active += !st->done[q];
      }
      st->all_done = active == 0;
   }
}

// mixed-precision helpers: r32 = r / ||r|| (zero where converged), x += ||r|| c
__global__ void blk_scale_kernel(int64_t n, int R, const double *r, const double *nrm2,
                                 const int *conv, float *r32)
{
   const int q = threadIdx.x % R;
   const double s = conv[q] ? 0.0 : 1.0 / sqrt(nrm2[q]);
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      r32[k] = (float)(r[k] * s);
   }
}
__global__ void blk_correct_kernel(int64_t n, int R, double *x, const float *c32,
                                   const double *nrm2, const int *conv)
{
   const int q = threadIdx.x % R;
   const double s = conv[q] ? 0.0 : sqrt(nrm2[q]);
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      x[k] += s * (double)c32[k];
   }
}
__global__ void blk_residual_kernel(int64_t n, const double *b, double *r)
{
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      r[k] = b[k] - r[k];
   }
}

// ------------------------------------------------------------ host side
static bool rhs_ok(int R) { return R == 1 || R == 2 || R == 4 || R == 8; }

// The tensor-core block apply's data for R vectors (FP32 symmetric diffusion
// with a block kernel for (D, Q, R), while that layout is selected): built
// once, outside any graph capture (every block path prepares its scratch
// before it captures).
static bool block_tc_wanted(const gbpa_operator *op, int R)
{
   const gbpa_operator_desc &d = op->d;
   return d.precision == GBPA_F32 && d.kind == GBPA_DIFFUSION && d.symm && tc::block_supported(d.d1d, d.q1d, R) &&
          block_apply_layout(d.d1d, d.q1d, R) == GBPA_LAYOUT_TC;
}

static int ensure_block_tc(gbpa_operator *op, int R)
{
   if (!block_tc_wanted(op, R) || (op->tcb && op->tcb_nrhs == R)) { return GBPA_SUCCESS; }
   const gbpa_operator_desc &d = op->d;
   if (op->tcb)
   {
      cudaStreamSynchronize(op->ctx->stream);
      tc::free_tables(op->tcb);
      delete op->tcb;
      op->tcb = nullptr;
      cudaFree(op->tcb_qdata);
      op->tcb_qdata = nullptr;
   }
   op->tcb_nrhs = 0;
   const int n = d.q1d * d.d1d;
   std::vector<float> bf(n), gf(n);
   int rc = check_cuda(cudaMemcpy(bf.data(), d.B, sizeof(float) * n, cudaMemcpyDeviceToHost), "copy B");
   if (!rc) { rc = check_cuda(cudaMemcpy(gf.data(), d.G, sizeof(float) * n, cudaMemcpyDeviceToHost), "copy G"); }
   if (rc) { return rc; }
   std::vector<double> bd(bf.begin(), bf.end()), gd(gf.begin(), gf.end());
   op->tcb = new (std::nothrow) tc::Tables;
   if (!op->tcb) { return GBPA_ERR_OUT_OF_MEMORY; }
   rc = tc::build_block_tables(d.d1d, d.q1d, bd.data(), gd.data(), op->tcb);
   if (!rc && !op->tcb_qscale)
   {
      rc = check_cuda(cudaMalloc(&op->tcb_qscale, sizeof(float) * d.ne), "cudaMalloc(tc block scale)");
   }
   if (!rc)
   {
      rc = tc::launch_qscale(op->ctx, d.ne, d.q1d, (const float *)d.qdata, (float)op->tcb->R, op->tcb_qscale);
   }
   if (!rc)
   {
      const int64_t nq = tc::block_qdata_size(d.d1d, d.q1d, R, d.ne);
      rc = check_cuda(cudaMalloc(&op->tcb_qdata, sizeof(float) * nq), "cudaMalloc(tc block qdata)");
   }
   if (!rc)
   {
      rc = tc::launch_block_transpose_qdata(op->ctx, d.ne, d.d1d, d.q1d, R, (const float *)d.qdata,
                                            op->tcb_qdata);
   }
   if (rc)
   {
      if (op->tcb) { tc::free_tables(op->tcb); delete op->tcb; op->tcb = nullptr; }
      cudaFree(op->tcb_qdata);
      op->tcb_qdata = nullptr;
      return rc;
   }
   op->tcb_nrhs = R;
   return GBPA_SUCCESS;
}

static int ensure_block_scratch(gbpa_operator *op, int R)
{
   const int rt = ensure_block_tc(op, R);
   if (rt) { return rt; }
   if (op->yEb && op->yEb_nrhs >= R) { return GBPA_SUCCESS; }
   cudaFree(op->yEb);
   op->yEb = nullptr;
   const int64_t nE = (int64_t)op->d.ne * op->d.d1d * op->d.d1d * op->d.d1d;
   const size_t w = op->d.precision == GBPA_F32 ? 4 : 8;
   const int rc = check_cuda(cudaMalloc(&op->yEb, w * nE * R + 256), "cudaMalloc(yE block)");
   op->yEb_nrhs = rc ? 0 : R;
   return rc;
}

template <typename T>
static int block_apply_evec(gbpa_operator *op, int R, const T *x, const int *skip)
{
   const gbpa_operator_desc &d = op->d;
   if (d.kind != GBPA_DIFFUSION) { return GBPA_ERR_UNSUPPORTED; }
   if constexpr (sizeof(T) == 4)
   {
      if (op->tcb && op->tcb_nrhs == R && block_tc_wanted(op, R))
      {
         return tc::launch_diffusion_block_f32(op->ctx, d.ne, d.d1d, d.q1d, R, *op->tcb, op->tcb_qdata,
                                               op->tcb_qscale, x, op->gather(), op->gather_mask(),
                                               (float *)op->yEb, skip);
      }
      return launch_diffusion_block_f32(op->ctx, d.ne, R, d.symm ? 1 : 0, d.d1d, d.q1d,
                                        (const float *)d.B, (const float *)d.G,
                                        (const float *)d.qdata, x, op->gather(), op->gather_mask(),
                                        (float *)op->yEb, skip);
   }
   else
   {
      return launch_diffusion_block_f64(op->ctx, d.ne, R, d.symm ? 1 : 0, d.d1d, d.q1d,
                                        (const double *)d.B, (const double *)d.G,
                                        (const double *)d.qdata, x, op->gather(), op->gather_mask(),
                                        (double *)op->yEb, skip);
   }
}

template <typename T>
static int block_mult(gbpa_operator *op, int R, const T *x, T *y)
{
   int rc = ensure_block_scratch(op, R);
   if (rc) { return rc; }
   rc = block_apply_evec<T>(op, R, x, nullptr);
   if (rc) { return rc; }
   const int64_t n = (int64_t)op->d.ndofs * R;
   const uintptr_t vec = (uintptr_t)(sizeof(T) * R);
   if (R > 1 && (uintptr_t)y % vec == 0 && (uintptr_t)x % vec == 0)
   {
      const unsigned grid = grid_for(op->d.ndofs, 256, 8 * op->ctx->num_sms);
      const int nd = op->d.ndofs;
      const T *yE = (const T *)op->yEb;
      cudaStream_t s = op->ctx->stream;
      switch (R)
      {
      case 2: blk_scatter_rhs_kernel<T, 2><<<grid, 256, 0, s>>>(nd, op->d.offsets, op->d.indices, yE, y, op->mask, x); break;
      case 4: blk_scatter_rhs_kernel<T, 4><<<grid, 256, 0, s>>>(nd, op->d.offsets, op->d.indices, yE, y, op->mask, x); break;
      default: blk_scatter_rhs_kernel<T, 8><<<grid, 256, 0, s>>>(nd, op->d.offsets, op->d.indices, yE, y, op->mask, x); break;
      }
      return last_launch(op->ctx, "blk_scatter_rhs");
   }
   blk_scatter_kernel<T><<<grid_for(n, 256), 256, 0, op->ctx->stream>>>(
      op->d.ndofs, R, op->d.offsets, op->d.indices, (const T *)op->yEb, y, op->mask, x);
   return last_launch(op->ctx, "blk_scatter");
}

template <typename T>
static int launch_scatter_den(gbpa_operator *op, int R, T *z, const T *d, double *partials,
                              BlockState *st, int first)
{
   gbpa_ctx *ctx = op->ctx;
   // 256 threads: the R = 8 variants hold 80-96 registers, three blocks per SM
   constexpr int BS = 256;
   const unsigned grid = grid_for(op->d.ndofs, BS, 8 * ctx->num_sms);
   const T *yE = (const T *)op->yEb;
   const gbpa_operator_desc &od = op->d;
   switch (R)
   {
   case 1: blk_scatter_den_kernel<T, 1><<<grid, BS, 0, ctx->stream>>>(od.ndofs, od.offsets, od.indices, yE, z, d, op->mask, partials, st, first); break;
   case 2: blk_scatter_den_kernel<T, 2><<<grid, BS, 0, ctx->stream>>>(od.ndofs, od.offsets, od.indices, yE, z, d, op->mask, partials, st, first); break;
   case 4: blk_scatter_den_kernel<T, 4><<<grid, BS, 0, ctx->stream>>>(od.ndofs, od.offsets, od.indices, yE, z, d, op->mask, partials, st, first); break;
   default: blk_scatter_den_kernel<T, 8><<<grid, BS, 0, ctx->stream>>>(od.ndofs, od.offsets, od.indices, yE, z, d, op->mask, partials, st, first); break;
   }
   return last_launch(ctx, "blk_scatter_den");
}

struct BlockWork
{
   void *r = nullptr, *d = nullptr, *z = nullptr;
   double *partials = nullptr;
   BlockState *st = nullptr;
   void free_all() { cudaFree(r); cudaFree(d); cudaFree(z); cudaFree(partials); cudaFree(st); }
};

// Block PCG iterations (update, direction, A d, den) in batches of K between
// host polls of the all-done flag, until every right-hand side is done.
template <typename T>
static int block_iterate(gbpa_operator *op, int R, T *x, T *r, T *z, T *d, const T *dinv,
                         BlockWork &w, int max_it)
{
   gbpa_ctx *ctx = op->ctx;
   const int64_t n = (int64_t)op->d.ndofs * R;
   const unsigned grid = grid_for(n, BK_BLOCK, 4 * ctx->num_sms);
   const int K = 10;
   int *h_done = (int *)ctx->h_pinned;
   int rc = GBPA_SUCCESS;
   for (int launched = 0; !rc; launched += K)
   {
      rc = check_cuda(cudaMemcpyAsync(h_done, &w.st->all_done, sizeof(int), cudaMemcpyDeviceToHost,
                                      ctx->stream), "copy");
      if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
      if (rc || *h_done || launched > max_it + K) { break; }
      for (int k = 0; k < K && !rc; ++k)
      {
         blk_update_kernel<T><<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, x, r, z, d, dinv, w.partials,
                                                                 w.st);
         rc = last_launch(ctx, "blk_update");
         if (!rc)
         {
            blk_direction_kernel<T><<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, z, d, w.st);
            rc = last_launch(ctx, "blk_direction");
         }
         if (!rc) { rc = block_apply_evec<T>(op, R, d, &w.st->all_done); }
         if (!rc)
         {
            rc = launch_scatter_den<T>(op, R, z, d, w.partials + 4096 * 4, w.st, 0);
         }
      }
   }
   return rc;
}

template <typename T>
static int block_pcg_run(gbpa_operator *op, int R, const T *dinv, const T *b, T *x,
                         double rel_tol, double abs_tol, int max_it, BlockState *h_out,
                         float *ms_out)
{
   gbpa_ctx *ctx = op->ctx;
   const int64_t n = (int64_t)op->d.ndofs * R;
   int rc = ensure_block_scratch(op, R);
   if (rc) { return rc; }
   BlockWork w;
   rc = check_cuda(cudaMalloc(&w.r, sizeof(T) * n), "cudaMalloc");
   if (!rc) { rc = check_cuda(cudaMalloc(&w.d, sizeof(T) * n), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&w.z, sizeof(T) * n), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&w.partials, sizeof(double) * 4096 * BK_MAXR), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&w.st, sizeof(BlockState)), "cudaMalloc"); }
   if (rc) { w.free_all(); return rc; }
   T *r = (T *)w.r, *d = (T *)w.d, *z = (T *)w.z;
   const unsigned grid = grid_for(n, BK_BLOCK, 4 * ctx->num_sms);
   BlockState h{};
   h.nrhs = R; h.max_it = max_it; h.rel2 = rel_tol * rel_tol; h.abs2 = abs_tol * abs_tol;
   StreamTimer timer(ctx->stream);
   rc = check_cuda(cudaMemcpyAsync(w.st, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream), "copy");
   if (!rc)
   {
      blk_init_kernel<T><<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, b, x, r, z, d, dinv, w.partials, w.st);
      rc = last_launch(ctx, "blk_init");
   }
   if (!rc) { rc = block_apply_evec<T>(op, R, d, &w.st->all_done); }
   if (!rc)
   {
      rc = launch_scatter_den<T>(op, R, z, d, w.partials + 4096 * 4, w.st, 1);
   }
   if (!rc) { rc = block_iterate<T>(op, R, x, r, z, d, dinv, w, max_it); }
   const float ms = timer.stop(ctx->stream);
   if (ms_out) { *ms_out = ms; }
   if (!rc) { rc = check_cuda(cudaMemcpy(h_out, w.st, sizeof(BlockState), cudaMemcpyDeviceToHost), "copy"); }
   w.free_all();
   if (rc) { return rc; }
   return h_out->status;
}

// out[q] = (a_q, b_q) for the R interleaved vectors, on the host
template <typename T>
static int block_dots(gbpa_ctx *ctx, int64_t n, int R, const T *a, const T *b, double *partials,
                      unsigned int *counter, double *d_out, double *h_out)
{
   const unsigned grid = grid_for(n, BK_BLOCK, 4 * ctx->num_sms);
   blk_dot_kernel<T><<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, a, b, partials, counter, d_out);
   int rc = last_launch(ctx, "blk_dot");
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(h_out, d_out, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy"); }
   if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
   return rc;
}

} // namespace gbpa

using namespace gbpa;

extern "C" int gbpa_operator_mult_block(gbpa_operator_t op, int nrhs, const void *x, void *y)
{
   if (!op || !rhs_ok(nrhs) || (op->d.ndofs > 0 && (!x || !y))) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (op->d.kind != GBPA_DIFFUSION) { return GBPA_ERR_UNSUPPORTED; }
   if (op->d.ndofs == 0) { return GBPA_SUCCESS; }
   if (op->d.precision == GBPA_F32) { return block_mult<float>(op, nrhs, (const float *)x, (float *)y); }
   return block_mult<double>(op, nrhs, (const double *)x, (double *)y);
}

static void fill_info(const BlockState &h, int R, float ms, gbpa_solve_info *info)
{
   for (int q = 0; q < R; ++q)
   {
      gbpa_solve_info &f = info[q];
      memset(&f, 0, sizeof(f));
      f.iterations = h.final_iter[q];
      f.converged = h.converged[q];
      f.initial_norm = h.nom0[q] >= 0 ? sqrt(h.nom0[q]) : h.nom0[q];
      f.final_norm = h.betanom[q] >= 0 ? sqrt(h.betanom[q]) : h.betanom[q];
      f.outer_iterations = 1;
      f.inner_iterations = h.final_iter[q];
      f.seconds = ms * 1e-3;
      f.true_rel_residual = -1.0;
   }
}

extern "C" int gbpa_pcg_solve_block(gbpa_operator_t A, int nrhs, const double *dinv, const double *b,
                                    double *x, double rel_tol, double abs_tol, int max_it,
                                    gbpa_solve_info *info)
{
   if (!A || !rhs_ok(nrhs) || !info || max_it < 0 || rel_tol < 0 || abs_tol < 0) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (A->d.precision == GBPA_F32 || A->d.kind != GBPA_DIFFUSION) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (A->d.ndofs == 0) { return GBPA_SUCCESS; }
   if (!dinv || !b || !x) { return GBPA_ERR_INVALID_ARGUMENT; }
   BlockState h{};
   float ms = 0.f;
   const int rc = block_pcg_run<double>(A, nrhs, dinv, b, x, rel_tol, abs_tol, max_it, &h, &ms);
   fill_info(h, nrhs, ms, info);
   return rc;
}

extern "C" int gbpa_pcg_solve_block_mixed(gbpa_operator_t A64, gbpa_operator_t A32, int nrhs,
                                          const float *dinv32, const double *b, double *x,
                                          double outer_rel_tol, double inner_rel_tol, int max_outer,
                                          int max_inner, gbpa_solve_info *info)
{
   if (!A64 || !A32 || !rhs_ok(nrhs) || !info || A64->d.precision == GBPA_F32 ||
       A32->d.precision != GBPA_F32 || A64->d.ndofs != A32->d.ndofs || A64->ctx != A32->ctx ||
       max_outer < 1 || max_inner < 1 || A64->d.kind != GBPA_DIFFUSION || A32->d.kind != GBPA_DIFFUSION)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   const int R = nrhs;
   const int64_t n = (int64_t)A64->d.ndofs * R;
   if (n == 0) { return GBPA_SUCCESS; }
   if (!dinv32 || !b || !x) { return GBPA_ERR_INVALID_ARGUMENT; }
   gbpa_ctx *ctx = A64->ctx;
   // FP64 residual, FP32 rhs/correction, reduction scratch
   double *r64 = nullptr, *red = nullptr;
   float *r32 = nullptr, *c32 = nullptr;
   int *conv_d = nullptr;
   int rc = check_cuda(cudaMalloc(&r64, sizeof(double) * n), "cudaMalloc");
   if (!rc) { rc = check_cuda(cudaMalloc(&r32, sizeof(float) * n), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&c32, sizeof(float) * n), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&red, sizeof(double) * (4096 * BK_MAXR + 64)), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&conv_d, sizeof(int) * BK_MAXR), "cudaMalloc"); }
   auto cleanup = [&]() { cudaFree(r64); cudaFree(r32); cudaFree(c32); cudaFree(red); cudaFree(conv_d); };
   if (rc) { cleanup(); return rc; }
   unsigned int *counter = (unsigned int *)(red + 4096 * BK_MAXR);
   double *d_out = red + 4096 * BK_MAXR + 16;
   cudaMemsetAsync(counter, 0, sizeof(unsigned int) * 4, ctx->stream);
   StreamTimer timer(ctx->stream);
   double nb2[BK_MAXR] = {0}, rn2[BK_MAXR] = {0};
   int conv[BK_MAXR] = {0}, outer_its[BK_MAXR] = {0}, inner_its[BK_MAXR] = {0};
   rc = check_cuda(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream), "memset");
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(r64, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream), "copy"); }
   if (!rc) { rc = block_dots<double>(ctx, n, R, b, b, red, counter, d_out, nb2); }
   int outer = 0;
   for (outer = 0; !rc && outer <= max_outer; ++outer)
   {
      rc = block_dots<double>(ctx, n, R, r64, r64, red, counter, d_out, rn2);
      if (rc) { break; }
      int all = 1;
      for (int q = 0; q < R; ++q)
      {
         if (!std::isfinite(rn2[q])) { rc = GBPA_ERR_NOT_FINITE; break; }
         const double rel = nb2[q] > 0 ? sqrt(rn2[q] / nb2[q]) : sqrt(rn2[q]);
         if (!conv[q] && rel <= outer_rel_tol) { conv[q] = 1; outer_its[q] = outer; }
         all &= conv[q];
      }
      if (rc || all || outer == max_outer) { break; }
      rc = check_cuda(cudaMemcpyAsync(conv_d, conv, sizeof(int) * R, cudaMemcpyHostToDevice, ctx->stream), "copy");
      if (rc) { break; }
      // device copy of ||r||^2 for the scale/correct kernels
      rc = check_cuda(cudaMemcpyAsync(d_out, rn2, sizeof(double) * R, cudaMemcpyHostToDevice, ctx->stream), "copy");
      if (rc) { break; }
      blk_scale_kernel<<<grid_for(n, BK_BLOCK, 4 * ctx->num_sms), BK_BLOCK, 0, ctx->stream>>>(n, R, r64, d_out, conv_d, r32);
      rc = last_launch(ctx, "blk_scale");
      if (rc) { break; }
      BlockState hs{};
      rc = block_pcg_run<float>(A32, R, dinv32, r32, c32, inner_rel_tol, 0.0, max_inner, &hs, nullptr);
      if (rc) { break; }
      for (int q = 0; q < R; ++q) { inner_its[q] += conv[q] ? 0 : hs.final_iter[q]; }
      rc = check_cuda(cudaMemcpyAsync(d_out, rn2, sizeof(double) * R, cudaMemcpyHostToDevice, ctx->stream), "copy");
      if (rc) { break; }
      blk_correct_kernel<<<grid_for(n, BK_BLOCK, 4 * ctx->num_sms), BK_BLOCK, 0, ctx->stream>>>(n, R, x, c32, d_out, conv_d);
      rc = last_launch(ctx, "blk_correct");
      if (!rc) { rc = block_mult<double>(A64, R, x, r64); }
      if (!rc)
      {
         blk_residual_kernel<<<grid_for(n, BK_BLOCK, 4 * ctx->num_sms), BK_BLOCK, 0, ctx->stream>>>(n, b, r64);
         rc = last_launch(ctx, "blk_residual");
      }
   }
   const float ms = timer.stop(ctx->stream);
   cleanup();
   int all = 1;
   for (int q = 0; q < R; ++q)
   {
      gbpa_solve_info &f = info[q];
      memset(&f, 0, sizeof(f));
      f.converged = conv[q];
      f.outer_iterations = conv[q] ? outer_its[q] : outer;
      f.inner_iterations = inner_its[q];
      f.iterations = inner_its[q];
      f.true_rel_residual = nb2[q] > 0 ? sqrt(rn2[q] / nb2[q]) : sqrt(rn2[q]);
      f.final_norm = sqrt(rn2[q]);
      f.seconds = ms * 1e-3;
      all &= conv[q];
   }
   if (rc) { return rc; }
   return all ? GBPA_SUCCESS : GBPA_ERR_NOT_CONVERGED;
}

// Block form of the reliable-update mixed solver: one FP32 block PCG on A32
// (each right-hand side scaled by 1/||b_r||) whose iterated residuals are
// replaced by the true FP64 block residual b - A64 x once every right-hand
// side still running has dropped its preconditioned residual by delta since
// its last replacement; search directions keep their history. Right-hand
// sides stop on their own true FP64 residual.
extern "C" int gbpa_pcg_solve_block_mixed_reliable(gbpa_operator_t A64, gbpa_operator_t A32, int nrhs,
                                                   const float *dinv32, const double *b, double *x,
                                                   double rel_tol, double delta, int max_it,
                                                   gbpa_solve_info *info)
{
   if (!A64 || !A32 || !rhs_ok(nrhs) || !info || A64->d.precision == GBPA_F32 ||
       A32->d.precision != GBPA_F32 || A64->d.ndofs != A32->d.ndofs || A64->ctx != A32->ctx ||
       max_it < 1 || rel_tol < 0 || !(delta > 0.0 && delta < 1.0) || A64->d.kind != GBPA_DIFFUSION ||
       A32->d.kind != GBPA_DIFFUSION)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   const int R = nrhs;
   const int64_t n = (int64_t)A64->d.ndofs * R;
   if (n == 0) { return GBPA_SUCCESS; }
   if (!dinv32 || !b || !x) { return GBPA_ERR_INVALID_ARGUMENT; }
   gbpa_ctx *ctx = A64->ctx;
   gbpa_operator *op = A32;
   int rc = ensure_block_scratch(op, R);
   if (rc) { return rc; }
   double *r64 = nullptr, *red = nullptr;
   float *b32 = nullptr, *x32 = nullptr;
   int *conv_d = nullptr;
   BlockWork w;
   rc = check_cuda(cudaMalloc(&r64, sizeof(double) * n), "cudaMalloc");
   if (!rc) { rc = check_cuda(cudaMalloc(&b32, sizeof(float) * n), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&x32, sizeof(float) * n), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&red, sizeof(double) * (4096 * BK_MAXR + 64)), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&conv_d, sizeof(int) * BK_MAXR), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&w.r, sizeof(float) * n), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&w.d, sizeof(float) * n), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&w.z, sizeof(float) * n), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&w.partials, sizeof(double) * 4096 * BK_MAXR), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&w.st, sizeof(BlockState)), "cudaMalloc"); }
   auto cleanup = [&]() {
      cudaFree(r64); cudaFree(b32); cudaFree(x32); cudaFree(red); cudaFree(conv_d); w.free_all();
   };
   if (rc) { cleanup(); return rc; }
   float *r = (float *)w.r, *d = (float *)w.d, *z = (float *)w.z;
   unsigned int *counter = (unsigned int *)(red + 4096 * BK_MAXR);
   double *d_out = red + 4096 * BK_MAXR + 16;
   double *d_nb2 = red + 4096 * BK_MAXR + 32;
   const unsigned grid = grid_for(n, BK_BLOCK, 4 * ctx->num_sms);
   StreamTimer timer(ctx->stream);
   double nb2[BK_MAXR] = {0}, rn2[BK_MAXR] = {0};
   int conv[BK_MAXR] = {0}, repl[BK_MAXR] = {0};
   BlockState hs{};
   rc = check_cuda(cudaMemsetAsync(counter, 0, sizeof(unsigned int) * 4, ctx->stream), "memset");
   if (!rc) { rc = check_cuda(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream), "memset"); }
   if (!rc) { rc = block_dots<double>(ctx, n, R, b, b, red, counter, d_out, nb2); }
   for (int q = 0; !rc && q < R; ++q)
   {
      if (!std::isfinite(nb2[q])) { rc = GBPA_ERR_NOT_FINITE; }
      conv[q] = nb2[q] == 0.0;   // b_r = 0: x_r = 0 is the solution
      if (conv[q]) { nb2[q] = 1.0; }
   }
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(d_nb2, nb2, sizeof(double) * R, cudaMemcpyHostToDevice, ctx->stream), "copy"); }
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(conv_d, conv, sizeof(int) * R, cudaMemcpyHostToDevice, ctx->stream), "copy"); }
   if (!rc)
   {
      // b32 = b_r / ||b_r|| (zero for a zero right-hand side)
      blk_scale_kernel<<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, b, d_nb2, conv_d, b32);
      rc = last_launch(ctx, "blk_scale");
   }
   if (!rc)
   {
      BlockState h{};
      h.nrhs = R; h.max_it = max_it; h.rel2 = delta * delta; h.abs2 = 0.0;
      rc = check_cuda(cudaMemcpyAsync(w.st, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream), "copy");
   }
   if (!rc)
   {
      blk_init_kernel<float><<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, b32, x32, r, z, d, dinv32, w.partials, w.st);
      rc = last_launch(ctx, "blk_init");
   }
   if (!rc) { rc = block_apply_evec<float>(op, R, d, &w.st->all_done); }
   if (!rc) { rc = launch_scatter_den<float>(op, R, z, d, w.partials + 4096 * 4, w.st, 1); }
   int all = 0;
   while (!rc)
   {
      rc = block_iterate<float>(op, R, x32, r, z, d, dinv32, w, max_it);
      if (!rc) { rc = check_cuda(cudaMemcpy(&hs, w.st, sizeof(BlockState), cudaMemcpyDeviceToHost), "copy"); }
      if (!rc && hs.status) { rc = hs.status; }
      if (rc) { break; }
      // replacement: x += ||b_r|| x32, x32 = 0, r64 = b - A64 x (FP64)
      blk_correct_kernel<<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, x, x32, d_nb2, conv_d);
      rc = last_launch(ctx, "blk_correct");
      if (!rc) { rc = check_cuda(cudaMemsetAsync(x32, 0, sizeof(float) * n, ctx->stream), "memset"); }
      if (!rc) { rc = block_mult<double>(A64, R, x, r64); }
      if (!rc)
      {
         blk_residual_kernel<<<grid, BK_BLOCK, 0, ctx->stream>>>(n, b, r64);
         rc = last_launch(ctx, "blk_residual");
      }
      if (!rc) { rc = block_dots<double>(ctx, n, R, r64, r64, red, counter, d_out, rn2); }
      if (rc) { break; }
      all = 1;
      int capped = 0;
      for (int q = 0; q < R; ++q)
      {
         if (!std::isfinite(rn2[q])) { rc = GBPA_ERR_NOT_FINITE; break; }
         if (!conv[q])
         {
            ++repl[q];
            if (sqrt(rn2[q] / nb2[q]) <= rel_tol) { conv[q] = 1; }
            else if (hs.iter[q] > max_it || (hs.done[q] && !hs.converged[q])) { capped = 1; }
         }
         all &= conv[q];
      }
      if (rc || all || capped) { break; }
      // r = r64_r / ||b_r|| (zero where converged); z, betanom, beta; directions continue
      rc = check_cuda(cudaMemcpyAsync(conv_d, conv, sizeof(int) * R, cudaMemcpyHostToDevice, ctx->stream), "copy");
      if (!rc)
      {
         blk_scale_kernel<<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, r64, d_nb2, conv_d, r);
         rc = last_launch(ctx, "blk_scale");
      }
      if (!rc)
      {
         blk_restart_kernel<<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, r, z, dinv32, conv_d, w.partials, w.st);
         rc = last_launch(ctx, "blk_restart");
      }
      if (!rc)
      {
         blk_direction_kernel<float><<<grid, BK_BLOCK, 0, ctx->stream>>>(n, R, z, d, w.st);
         rc = last_launch(ctx, "blk_direction");
      }
      if (!rc) { rc = block_apply_evec<float>(op, R, d, &w.st->all_done); }
      if (!rc) { rc = launch_scatter_den<float>(op, R, z, d, w.partials + 4096 * 4, w.st, 0); }
   }
   const float ms = timer.stop(ctx->stream);
   cleanup();
   for (int q = 0; q < R; ++q)
   {
      gbpa_solve_info &f = info[q];
      memset(&f, 0, sizeof(f));
      f.converged = conv[q];
      f.outer_iterations = repl[q];
      f.inner_iterations = hs.iter[q];
      f.iterations = hs.iter[q];
      f.true_rel_residual = sqrt(rn2[q] / nb2[q]);
      f.final_norm = sqrt(rn2[q]);
      f.seconds = ms * 1e-3;
   }
   if (rc) { return rc; }
   return all ? GBPA_SUCCESS : GBPA_ERR_NOT_CONVERGED;
}
