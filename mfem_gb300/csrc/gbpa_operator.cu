// L-vector PA operator (restriction + integrator + transpose, optionally
// constrained), its diagonal, and the device-resident PCG solvers.
//   PABilinearFormExtension::Mult     fem/bilinearform_ext.cpp:487-564
//   PABilinearFormExtension::AssembleDiagonal  fem/bilinearform_ext.cpp:370-454
//   ConstrainedOperator (DIAG_ONE)    linalg/operator.cpp:526-661
//   CGSolver::Mult                    linalg/solvers.cpp:869-1050
//   OperatorJacobiSmoother::Mult      linalg/solvers.cpp:427-452
#include "gbpa_csr.cuh"
#include "gbpa_operator.cuh"
#include <type_traits>
#include <vector>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>

namespace gbpa
{
constexpr int PCG_BLOCK = 512;

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) { v += __shfl_down_sync(0xffffffffu, v, o); }
   return v;
}

// Block sum; result valid in thread 0. Uses a caller-provided 32-entry buffer.
__device__ double block_sum_d(double v, double *ws)
{
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   v = warp_sum_d(v);
   if (lane == 0) { ws[wid] = v; }
   __syncthreads();
   const int nw = (blockDim.x + 31) >> 5;
   v = threadIdx.x < nw ? ws[threadIdx.x] : 0.0;
   if (wid == 0) { v = warp_sum_d(v); }
   __syncthreads();
   return v;
}

// Publishes this block's partial and returns true in the last block to
// arrive (which then sees every partial). Deterministic: the last block sums
// partials in block order.
__device__ bool finish_partial(double s, double *partials, unsigned int *counter,
                               double *total, double *ws)
{
   __shared__ bool last;
   if (threadIdx.x == 0)
   {
      partials[blockIdx.x] = s;
      __threadfence();
      last = atomicInc(counter, gridDim.x - 1) == gridDim.x - 1;
   }
   __syncthreads();
   if (!last) { return false; }
   __threadfence();
   double t = 0.0;
   for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
   {
      t += ((volatile double *)partials)[b];
   }
   t = block_sum_d(t, ws);
   if (threadIdx.x == 0) { *total = t; }
   return true;
}

// init: x = 0 (unless iterative), r = b or r = b - Ax (r holds Ax on entry),
// z = dinv r, d = z, nom = (d, r)
template <typename T>
__global__ void pcg_init_kernel(int64_t n, const T *__restrict__ b, T *__restrict__ x,
                                T *__restrict__ r, T *__restrict__ z, T *__restrict__ d,
                                const T *__restrict__ dinv, int iterative,
                                double *partials, PcgState *st)
{
   __shared__ double ws[32];
   double s = 0.0;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      T ri;
      if (iterative) { ri = b[i] - r[i]; }
      else { ri = b[i]; x[i] = T(0); }
      r[i] = ri;
      const T zi = dinv[i] * ri;
      z[i] = zi;
      d[i] = zi;
      s += (double)zi * (double)ri;
   }
   s = block_sum_d(s, ws);
   double tot;
   if (finish_partial(s, partials, &st->counter_init, &tot, ws) && threadIdx.x == 0)
   {
      st->nom = st->nom0 = tot;
      st->iter = 1;
      st->converged = 0;
      st->status = 0;
      st->final_iter = 0;
      st->done = 0;
      st->betanom = tot;
      if (!isfinite(tot)) { st->status = GBPA_ERR_NOT_FINITE; st->done = 1; }
      else if (tot < 0.0) { st->done = 1; }
      else
      {
         st->r0 = fmax(tot * st->rel_tol2, st->abs_tol2);
         if (tot <= st->r0) { st->converged = 1; st->done = 1; }
      }
   }
}

// z = CSR scatter of yE (with constraint z[ess] = d[ess]); den = (d, z);
// then alpha = nom / den (and nom = betanom after the first iteration).
template <typename T>
__global__ void pcg_scatter_den_kernel(int ndofs, const int *__restrict__ offsets,
                                       const int *__restrict__ indices,
                                       const T *__restrict__ yE, T *__restrict__ z,
                                       const T *__restrict__ d,
                                       const unsigned char *__restrict__ mask,
                                       double *partials, PcgState *st, int first)
{
   if (st->done) { return; }
   __shared__ double ws[32];
   double s = 0.0;
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndofs; i += gridDim.x * blockDim.x)
   {
      T v;
      if (mask && mask[i]) { v = d[i]; }
      else if (offsets) { v = csr_row_sum<T>(offsets, indices, yE, i); }
      else { v = z[i]; }   // summed into z by the apply's atomic scatter
      z[i] = v;
      s += (double)d[i] * (double)v;
   }
   s = block_sum_d(s, ws);
   double den;
   if (finish_partial(s, partials, &st->counter_den, &den, ws) && threadIdx.x == 0)
   {
      st->den = den;
      if (!isfinite(den)) { st->status = GBPA_ERR_NOT_FINITE; st->done = 1; st->final_iter = st->iter; }
      else if (den == 0.0) { st->done = 1; st->final_iter = st->iter; }
      else
      {
         if (!first) { st->nom = st->betanom; }
         st->alpha = st->nom / den;
      }
   }
}

// x += alpha d; r -= alpha z; z = dinv r; betanom = (r, z); stopping test;
// beta = betanom / nom.
template <typename T>
__global__ void pcg_update_kernel(int64_t n, T *__restrict__ x, T *__restrict__ r,
                                  T *__restrict__ z, const T *__restrict__ d,
                                  const T *__restrict__ dinv, double *partials, PcgState *st)
{
   if (st->done) { return; }
   __shared__ double ws[32];
   const T alpha = (T)st->alpha;
   double s = 0.0;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      x[i] += alpha * d[i];
      const T ri = r[i] - alpha * z[i];
      r[i] = ri;
      const T zi = dinv[i] * ri;
      z[i] = zi;
      s += (double)ri * (double)zi;
   }
   s = block_sum_d(s, ws);
   double bn;
   if (finish_partial(s, partials, &st->counter_beta, &bn, ws) && threadIdx.x == 0)
   {
      st->betanom = bn;
      if (!isfinite(bn)) { st->status = GBPA_ERR_NOT_FINITE; st->done = 1; st->final_iter = st->iter; }
      else if (bn < 0.0) { st->done = 1; st->final_iter = st->iter; }
      else if (bn <= st->r0) { st->converged = 1; st->done = 1; st->final_iter = st->iter; }
      else if (++st->iter > st->max_it) { st->done = 1; st->final_iter = st->max_it; }
      else { st->beta = bn / st->nom; }
   }
}

// d = z + beta d
template <typename T>
__global__ void pcg_direction_kernel(int64_t n, const T *__restrict__ z, T *__restrict__ d,
                                     const PcgState *st)
{
   if (st->done) { return; }
   const T beta = (T)st->beta;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      d[i] = z[i] + beta * d[i];
   }
}

__global__ void fill_mask_kernel(int n, const int *ess, unsigned char *mask, int ndofs, int *flags)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
   {
      const int k = ess[i];
      if (k < 0 || k >= ndofs) { atomicOr(flags, GBPA_FLAG_INDEX); continue; }
      mask[k] = 1;
   }
}

// y[i] = x[i] on constrained dofs (ConstrainedOperator::Mult, after the
// atomic scatter left them zero)
template <typename T>
__global__ void copy_masked_kernel(int64_t n, const unsigned char *__restrict__ mask,
                                   const T *__restrict__ x, T *__restrict__ y)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      if (mask[i]) { y[i] = x[i]; }
   }
}

// Element markers (PABilinearFormExtension::AddMultWithMarkers /
// AddWithMarkers_, fem/bilinearform_ext.cpp:753-774,807-847): element e
// contributes iff its attribute a > 0 and markers[a - 1] != 0. An attribute
// past the marker array is an index error here (the reference reads past it).
__global__ void element_markers_kernel(int ne, const int *__restrict__ attributes,
                                       const int *__restrict__ markers, int n_markers,
                                       unsigned char *__restrict__ active, int *flags)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x)
   {
      const int a = attributes[e];
      if (a > n_markers) { atomicOr(flags, GBPA_FLAG_INDEX); active[e] = 0; continue; }
      active[e] = (a > 0 && markers[a - 1] != 0) ? 1 : 0;
   }
}

// The element kernels' gather map: GBPA_GATHER_SKIP on every slot whose dof is
// essential (mask) or whose element is unmarked (active); an unmarked element
// then gathers zeros, and its apply contributes exactly zero to the scatter.
__global__ void operator_gather_map_kernel(int64_t n, int nd, const int *__restrict__ gmap,
                                           const unsigned char *__restrict__ mask,
                                           const unsigned char *__restrict__ active,
                                           int *__restrict__ out)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int g = gmap[i];
      const int j = g >= 0 ? g : -1 - g;
      const bool off = (active && !active[i / nd]) || (mask && mask[j]);
      out[i] = off ? GBPA_GATHER_SKIP : g;
   }
}

// zero the E-vector entries of unmarked elements (diagonal with markers)
__global__ void zero_unmarked_kernel(int64_t n, int nd, const unsigned char *__restrict__ active,
                                     double *__restrict__ yE)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      if (!active[i / nd]) { yE[i] = 0.0; }
   }
}

__global__ void set_mask_one_kernel(int ndofs, const unsigned char *mask, double *y)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndofs; i += gridDim.x * blockDim.x)
   {
      if (mask[i]) { y[i] = 1.0; }
   }
}

// Reliable update of the FP32 CG (residual replaced by the true one, r
// already written): z = dinv r, betanom = (r, z), beta = betanom / nom (the
// direction keeps its history), and the next segment's stopping level
// r0 = rel_tol2 * betanom (rel_tol2 holds delta^2).
__global__ void pcg_restart_kernel(int64_t n, const float *__restrict__ r, float *__restrict__ z,
                                   const float *__restrict__ dinv, double *partials, PcgState *st)
{
   __shared__ double ws[32];
   double s = 0.0;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const float zi = dinv[i] * r[i];
      z[i] = zi;
      s += (double)r[i] * (double)zi;
   }
   s = block_sum_d(s, ws);
   double bn;
   if (finish_partial(s, partials, &st->counter_init, &bn, ws) && threadIdx.x == 0)
   {
      st->betanom = bn;
      st->converged = 0;
      st->done = 0;
      if (!isfinite(bn)) { st->status = GBPA_ERR_NOT_FINITE; st->done = 1; st->final_iter = st->iter; }
      else if (bn <= 0.0) { st->done = 1; st->final_iter = st->iter; }
      else
      {
         st->beta = bn / st->nom;
         st->r0 = st->rel_tol2 * bn;
      }
   }
}

// mixed-precision helpers
__global__ void scale_to_f32_kernel(int64_t n, const double *r, const double *nrm2, float *r32)
{
   const double s = 1.0 / sqrt(*nrm2);
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      r32[i] = (float)(r[i] * s);
   }
}
__global__ void correct_kernel(int64_t n, double *x, const float *c32, const double *nrm2)
{
   const double s = sqrt(*nrm2);
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      x[i] += s * (double)c32[i];
   }
}
__global__ void residual_kernel(int64_t n, const double *b, double *r)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      r[i] = b[i] - r[i];
   }
}

} // namespace gbpa

using namespace gbpa;

static int64_t evec_size(const gbpa_operator_desc &d)
{
   return (int64_t)d.ne * d.d1d * d.d1d * d.d1d;
}
static size_t elem_bytes(const gbpa_operator_desc &d) { return d.precision == GBPA_F32 ? 4 : 8; }
static int64_t qdata_size(const gbpa_operator_desc &d)
{
   const int64_t q3 = (int64_t)d.q1d * d.q1d * d.q1d;
   return (int64_t)d.ne * q3 * (d.kind == GBPA_DIFFUSION ? (d.symm ? 6 : 9) : 1);
}

// Tensor-core layout of an FP32 diffusion operator: the Kronecker tables of
// its (FP32) basis tables and the per-element output scales.
static int setup_tensor_core(gbpa_operator *op)
{
   const gbpa_operator_desc &d = op->d;
   const int n = d.q1d * d.d1d;
   std::vector<float> bf(n), gf(n);
   int rc = check_cuda(cudaMemcpy(bf.data(), d.B, sizeof(float) * n, cudaMemcpyDeviceToHost), "copy B");
   if (!rc) { rc = check_cuda(cudaMemcpy(gf.data(), d.G, sizeof(float) * n, cudaMemcpyDeviceToHost), "copy G"); }
   if (rc) { return rc; }
   std::vector<double> bd(bf.begin(), bf.end()), gd(gf.begin(), gf.end());
   op->tct = new (std::nothrow) tc::Tables;
   if (!op->tct) { return GBPA_ERR_OUT_OF_MEMORY; }
   rc = tc::build_tables(d.d1d, d.q1d, bd.data(), gd.data(), op->tct);
   if (!rc) { rc = check_cuda(cudaMalloc(&op->tc_qscale, sizeof(float) * d.ne), "cudaMalloc(tc scale)"); }
   if (!rc)
   {
      rc = tc::launch_qscale(op->ctx, d.ne, d.q1d, (const float *)d.qdata, (float)op->tct->R, op->tc_qscale);
   }
   if (!rc)
   {
      const int64_t n = tc::transposed_qdata_size(d.d1d, d.q1d, d.ne);
      rc = check_cuda(cudaMalloc(&op->tc_qdata, sizeof(float) * n), "cudaMalloc(tc qdata)");
   }
   if (!rc) { rc = tc::launch_transpose_qdata(op->ctx, d.ne, d.d1d, d.q1d, (const float *)d.qdata, op->tc_qdata); }
   return rc;
}

extern "C" int gbpa_operator_create(gbpa_ctx_t ctx, const gbpa_operator_desc *desc,
                                    gbpa_operator_t *out)
{
   if (!ctx || !desc || !out) { return GBPA_ERR_INVALID_ARGUMENT; }
   *out = nullptr;
   const gbpa_operator_desc &d = *desc;
   if (d.kind != GBPA_DIFFUSION && d.kind != GBPA_MASS) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (d.precision != GBPA_F64 && d.precision != GBPA_F32 && d.precision != GBPA_F64X2)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (d.ne < 0 || d.ndofs < 0 || d.n_ess < 0) { return GBPA_ERR_INVALID_ARGUMENT; }
   // the double-float kernels are built for D1D, Q1D <= 10 (p <= 9)
   if (d.precision == GBPA_F64X2 && (d.d1d > 10 || d.q1d > 10)) { return GBPA_ERR_UNSUPPORTED; }
   if (d.d1d < 1 || d.q1d < 1 || d.d1d > GBPA_MAX_1D || d.q1d > GBPA_MAX_1D) { return GBPA_ERR_UNSUPPORTED; }
   if (d.ne > 0 && (!d.B || !d.qdata || !d.gather_map || !d.offsets || !d.indices)) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (d.kind == GBPA_DIFFUSION && d.ne > 0 && !d.G) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (d.n_ess > 0 && !d.ess) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (d.scatter != GBPA_SCATTER_CSR && d.scatter != GBPA_SCATTER_ATOMIC) { return GBPA_ERR_INVALID_ARGUMENT; }
   gbpa_operator *op = new (std::nothrow) gbpa_operator;
   if (!op) { return GBPA_ERR_OUT_OF_MEMORY; }
   op->ctx = ctx;
   op->d = d;
   int rc = GBPA_SUCCESS;
   const int64_t nE = evec_size(d);
   if (nE > 0) { rc = check_cuda(cudaMalloc(&op->yE, elem_bytes(d) * nE), "cudaMalloc(yE)"); }
   if (!rc && d.precision == GBPA_F64X2 && d.ne > 0)
   {
      const int64_t nq = qdata_size(d);
      rc = check_cuda(cudaMalloc(&op->qd2, sizeof(float2) * nq), "cudaMalloc(qdata x2)");
      if (!rc) { rc = launch_split_x2(ctx, nq, (const double *)d.qdata, op->qd2); }
   }
   if (!rc && d.n_ess > 0)
   {
      rc = check_cuda(cudaMalloc(&op->mask, d.ndofs), "cudaMalloc(mask)");
      if (!rc) { rc = check_cuda(cudaMemsetAsync(op->mask, 0, d.ndofs, ctx->stream), "memset"); }
      if (!rc)
      {
         fill_mask_kernel<<<grid_for(d.n_ess, 256), 256, 0, ctx->stream>>>(d.n_ess, d.ess, op->mask,
                                                                         d.ndofs, ctx->d_flags);
         rc = last_launch(ctx, "fill_mask");
      }
      int flags = 0;
      if (!rc) { rc = gbpa_get_error_flags(ctx, &flags); }
      if (!rc && (flags & GBPA_FLAG_INDEX)) { rc = GBPA_ERR_INDEX; }
      if (!rc && nE > 0)
      {
         rc = check_cuda(cudaMalloc(&op->gmap_m, sizeof(int) * nE), "cudaMalloc(masked map)");
         if (!rc) { rc = launch_masked_gather_map(ctx, nE, d.gather_map, op->mask, op->gmap_m); }
      }
   }
   if (!rc && d.kind == GBPA_DIFFUSION && d.precision == GBPA_F32 && d.symm && d.ne > 0 &&
       tc::supported(d.d1d, d.q1d) && apply_layout(GBPA_DIFFUSION, GBPA_F32, d.d1d, d.q1d, nullptr) == GBPA_LAYOUT_TC)
   {
      rc = setup_tensor_core(op);
   }
   if (rc) { gbpa_operator_destroy(op); return rc; }
   *out = op;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_operator_set_element_markers(gbpa_operator_t op, const int *attributes,
                                                 const int *markers, int n_markers)
{
   if (!op || n_markers < 0 || (attributes && n_markers > 0 && !markers)) { return GBPA_ERR_INVALID_ARGUMENT; }
   const gbpa_operator_desc &d = op->d;
   gbpa_ctx *ctx = op->ctx;
   const int64_t nE = evec_size(d);
   const int nd = d.d1d * d.d1d * d.d1d;
   // the element kernels' map changes: a captured PCG iteration is stale
   if (op->graph) { cudaStreamSynchronize(ctx->stream); cudaGraphExecDestroy(op->graph); op->graph = nullptr; }
   int rc = GBPA_SUCCESS;
   if (!attributes)
   {
      // back to every element
      cudaStreamSynchronize(ctx->stream);
      cudaFree(op->emask);
      op->emask = nullptr;
      if (!op->mask) { cudaFree(op->gmap_m); op->gmap_m = nullptr; return GBPA_SUCCESS; }
   }
   else if (d.ne > 0)
   {
      int flags = 0;
      rc = gbpa_get_error_flags(ctx, &flags);   // clear stale flags
      if (!rc && !op->emask) { rc = check_cuda(cudaMalloc(&op->emask, d.ne), "cudaMalloc(element markers)"); }
      if (!rc)
      {
         element_markers_kernel<<<grid_for(d.ne, 256), 256, 0, ctx->stream>>>(d.ne, attributes, markers, n_markers,
                                                                            op->emask, ctx->d_flags);
         rc = last_launch(ctx, "element_markers");
      }
      if (!rc) { rc = gbpa_get_error_flags(ctx, &flags); }
      if (!rc && (flags & GBPA_FLAG_INDEX)) { rc = GBPA_ERR_INDEX; }
      if (rc)
      {
         // refused: every element active again
         cudaStreamSynchronize(ctx->stream);
         cudaFree(op->emask);
         op->emask = nullptr;
         if (!op->mask) { cudaFree(op->gmap_m); op->gmap_m = nullptr; return rc; }
      }
   }
   if (nE == 0) { return rc; }
   if (!op->gmap_m)
   {
      const int ra = check_cuda(cudaMalloc(&op->gmap_m, sizeof(int) * nE), "cudaMalloc(masked map)");
      if (ra) { op->gmap_m = nullptr; return ra; }
   }
   operator_gather_map_kernel<<<grid_for(nE, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(
      nE, nd, d.gather_map, op->mask, op->emask, op->gmap_m);
   const int rl = last_launch(ctx, "operator_gather_map");
   return rc ? rc : rl;
}

// The descriptor's arrays in host memory: one device block holds copies of
// them (freed with the operator), then the operator is created on the copies.
extern "C" int gbpa_operator_create_host(gbpa_ctx_t ctx, const gbpa_operator_desc *desc, gbpa_operator_t *out)
{
   if (!ctx || !desc || !out) { return GBPA_ERR_INVALID_ARGUMENT; }
   *out = nullptr;
   const gbpa_operator_desc &d = *desc;
   if (d.ne < 0 || d.ndofs < 0 || d.n_ess < 0 || d.d1d < 1 || d.q1d < 1 ||
       (d.kind != GBPA_DIFFUSION && d.kind != GBPA_MASS) ||
       (d.precision != GBPA_F64 && d.precision != GBPA_F32 && d.precision != GBPA_F64X2))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   const size_t w = elem_bytes(d);
   const size_t nE = (size_t)evec_size(d);
   const size_t sizes[7] = {w * d.q1d * d.d1d, w * d.q1d * d.d1d, w * (size_t)qdata_size(d), sizeof(int) * nE,
                            sizeof(int) * ((size_t)d.ndofs + 1), sizeof(int) * nE, sizeof(int) * (size_t)d.n_ess};
   const void *src[7] = {d.B, d.G, d.qdata, d.gather_map, d.offsets, d.indices, d.ess};
   for (int k = 0; k < 7; ++k)
   {
      if (sizes[k] && !src[k] && k != 6) { return GBPA_ERR_INVALID_ARGUMENT; }
   }
   size_t off[7], total = 0;
   for (int k = 0; k < 7; ++k)
   {
      off[k] = total;
      total += (sizes[k] + 255) / 256 * 256;
   }
   unsigned char *blk = nullptr;
   int rc = check_cuda(cudaMalloc(&blk, total ? total : 256), "cudaMalloc(host operator copies)");
   for (int k = 0; k < 7 && !rc; ++k)
   {
      if (sizes[k] && src[k])
      {
         rc = check_cuda(cudaMemcpy(blk + off[k], src[k], sizes[k], cudaMemcpyHostToDevice), "copy operator array");
      }
   }
   if (rc) { cudaFree(blk); return rc; }
   gbpa_operator_desc dd = d;
   dd.B = blk + off[0];
   dd.G = blk + off[1];
   dd.qdata = blk + off[2];
   dd.gather_map = (const int *)(blk + off[3]);
   dd.offsets = (const int *)(blk + off[4]);
   dd.indices = (const int *)(blk + off[5]);
   dd.ess = d.n_ess > 0 && d.ess ? (const int *)(blk + off[6]) : nullptr;
   rc = gbpa_operator_create(ctx, &dd, out);
   if (rc) { cudaFree(blk); return rc; }
   (*out)->owned = blk;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_operator_destroy(gbpa_operator_t op)
{
   if (!op) { return GBPA_SUCCESS; }
   cudaStreamSynchronize(op->ctx->stream);
   if (op->graph) { cudaGraphExecDestroy(op->graph); }
   cudaFree(op->yE); cudaFree(op->mask); cudaFree(op->emask); cudaFree(op->gmap_m); cudaFree(op->qd2);
   cudaFree(op->r); cudaFree(op->dv); cudaFree(op->z);
   cudaFree(op->partials); cudaFree(op->state);
   cudaFree(op->r64); cudaFree(op->t64); cudaFree(op->yEb); cudaFree(op->stage);
   if (op->tct) { tc::free_tables(op->tct); delete op->tct; }
   cudaFree(op->tc_qscale);
   cudaFree(op->tc_qdata);
   if (op->tcb) { tc::free_tables(op->tcb); delete op->tcb; }
   cudaFree(op->tcb_qscale);
   cudaFree(op->tcb_qdata);
   cudaFree(op->owned);
   delete op;
   return GBPA_SUCCESS;
}

// out = A_e (R x) with the gather fused (ess dofs read as zero): the E-vector
// (mode 0), or with GBPA_OUT_ATOMIC the L-vector R^T A_e R x summed by atomics
// in the apply itself (out zeroed by the caller).
template <typename T>
static int apply_to(gbpa_operator *op, const T *x, T *out, int mode, const int *skip)
{
   const gbpa_operator_desc &d = op->d;
   if (d.precision == GBPA_F64X2)
   {
      const double *xd = (const double *)x;
      if (d.kind == GBPA_DIFFUSION)
      {
         return launch_diffusion_apply_x2(op->ctx, d.ne, d.symm ? 1 : 0, d.d1d, d.q1d,
                                          (const double *)d.B, (const double *)d.G, op->qd2, xd,
                                          op->gather(), op->gather_mask(), (double *)out, mode, skip);
      }
      return launch_mass_apply_x2(op->ctx, d.ne, d.d1d, d.q1d, (const double *)d.B, op->qd2, xd,
                                  op->gather(), op->gather_mask(), (double *)out, mode, skip);
   }
   if constexpr (std::is_same<T, float>::value)
   {
      // the tensor-core layout, while it stays selected for this order
      if (op->tct && apply_layout(GBPA_DIFFUSION, GBPA_F32, d.d1d, d.q1d, nullptr) == GBPA_LAYOUT_TC)
      {
         return tc::launch_diffusion_f32(op->ctx, d.ne, d.d1d, d.q1d, *op->tct, op->tc_qdata,
                                         op->tc_qscale, x, op->gather(), op->gather_mask(), out, mode, skip);
      }
   }
   if (d.kind == GBPA_DIFFUSION)
   {
      return launch_diffusion_apply<T>(op->ctx, d.ne, d.symm ? 1 : 0, d.d1d, d.q1d,
                                       (const T *)d.B, (const T *)d.G, (const T *)d.qdata, x,
                                       op->gather(), op->gather_mask(), out, mode, skip);
   }
   return launch_mass_apply<T>(op->ctx, d.ne, d.d1d, d.q1d, (const T *)d.B,
                               (const T *)d.qdata, x, op->gather(), op->gather_mask(), out, mode,
                               skip);
}

template <typename T>
static int apply_evec(gbpa_operator *op, const T *x, const int *skip)
{
   return apply_to<T>(op, x, (T *)op->yE, 0, skip);
}

static bool atomic_scatter(const gbpa_operator *op) { return op->d.scatter == GBPA_SCATTER_ATOMIC; }

template <typename T>
static int op_mult(gbpa_operator *op, const T *x, T *y)
{
   gbpa_ctx *ctx = op->ctx;
   if (atomic_scatter(op))
   {
      // y = R^T A_e R x by atomics inside the apply, then y[ess] = x[ess]
      const int64_t n = op->d.ndofs;
      int rc = check_cuda(cudaMemsetAsync(y, 0, sizeof(T) * n, ctx->stream), "memset(y)");
      if (!rc) { rc = apply_to<T>(op, x, y, GBPA_OUT_ATOMIC, nullptr); }
      if (!rc && op->mask)
      {
         copy_masked_kernel<T><<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(n, op->mask, x, y);
         rc = last_launch(ctx, "copy_masked");
      }
      return rc;
   }
   int rc = apply_evec<T>(op, x, nullptr);
   if (rc) { return rc; }
   return launch_csr_scatter<T>(ctx, op->d.ndofs, op->d.offsets, op->d.indices,
                                (const T *)op->yE, y, op->mask, x, false, false);
}

extern "C" int gbpa_operator_mult(gbpa_operator_t op, const void *x, void *y)
{
   if (!op || (op->d.ndofs > 0 && (!x || !y))) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (atomic_scatter(op) && x == y) { return GBPA_ERR_INVALID_ARGUMENT; }   // y is summed while x is read
   if (op->d.ndofs == 0) { return GBPA_SUCCESS; }
   if (op->d.precision != GBPA_F32) { return op_mult<double>(op, (const double *)x, (double *)y); }
   return op_mult<float>(op, (const float *)x, (float *)y);
}

// Device address of a host buffer the kernels can access directly: memory
// pinned by cudaHostAlloc / cudaHostRegister (device-mapped under unified
// addressing). Pageable memory returns nullptr, and so does any other kind
// (managed, device), which the caller then stages with cudaMemcpyDefault.
static void *mapped_host_ptr(const void *p)
{
   cudaPointerAttributes a{};
   if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
   {
      cudaGetLastError();   // an unregistered pointer is not an error here
      return nullptr;
   }
   return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

extern "C" int gbpa_operator_mult_host(gbpa_operator_t op, const void *x, void *y)
{
   if (!op || (op->d.ndofs > 0 && (!x || !y))) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (op->d.ndofs == 0) { return GBPA_SUCCESS; }
   gbpa_ctx *ctx = op->ctx;
   const size_t bytes = (size_t)op->d.ndofs * (op->d.precision == GBPA_F32 ? 4 : 8);
   void *dx = mapped_host_ptr(x), *dy = mapped_host_ptr(y);
   const bool stage_x = !dx, stage_y = !dy;
   int rc = GBPA_SUCCESS;
   if ((stage_x || stage_y) && !op->stage)
   {
      rc = check_cuda(cudaMalloc(&op->stage, 2 * bytes), "cudaMalloc(host staging)");
      if (rc) { op->stage = nullptr; return rc; }
   }
   if (stage_x)
   {
      dx = op->stage;
      rc = check_cuda(cudaMemcpyAsync(dx, x, bytes, cudaMemcpyDefault, ctx->stream), "copy x");
   }
   if (stage_y) { dy = (unsigned char *)op->stage + bytes; }
   if (!rc) { rc = gbpa_operator_mult(op, dx, dy); }
   if (!rc && stage_y)
   {
      rc = check_cuda(cudaMemcpyAsync(y, dy, bytes, cudaMemcpyDefault, ctx->stream), "copy y");
   }
   const int rs = check_cuda(cudaStreamSynchronize(ctx->stream), "sync");
   return rc ? rc : rs;
}

extern "C" int gbpa_operator_apply_element(gbpa_operator_t op, const void *x, void *yE)
{
   if (!op || (op->d.ne > 0 && (!x || !yE))) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (op->d.ne == 0) { return GBPA_SUCCESS; }
   void *saved = op->yE;
   op->yE = yE;
   const int rc = op->d.precision != GBPA_F32 ? apply_evec<double>(op, (const double *)x, nullptr)
                                              : apply_evec<float>(op, (const float *)x, nullptr);
   op->yE = saved;
   return rc;
}

extern "C" int gbpa_operator_assemble_diagonal(gbpa_operator_t op, double *diag)
{
   if (!op || (op->d.ndofs > 0 && !diag)) { return GBPA_ERR_INVALID_ARGUMENT; }
   const gbpa_operator_desc &d = op->d;
   if (d.ndofs == 0) { return GBPA_SUCCESS; }
   if (d.precision == GBPA_F32) { return GBPA_ERR_UNSUPPORTED; }
   gbpa_ctx *ctx = op->ctx;
   const int64_t nE = evec_size(d);
   int rc = check_cuda(cudaMemsetAsync(op->yE, 0, sizeof(double) * nE, ctx->stream), "memset");
   if (rc) { return rc; }
   if (d.kind == GBPA_DIFFUSION)
   {
      rc = launch_diffusion_diagonal(ctx, d.ne, d.symm ? 1 : 0, d.d1d, d.q1d, (const double *)d.B,
                                     (const double *)d.G, (const double *)d.qdata, (double *)op->yE);
   }
   else
   {
      rc = launch_mass_diagonal(ctx, d.ne, d.d1d, d.q1d, (const double *)d.B,
                                (const double *)d.qdata, (double *)op->yE);
   }
   if (rc) { return rc; }
   if (op->emask)
   {
      // assemble_diagonal_with_markers (fem/bilinearform_ext.cpp:405-440)
      zero_unmarked_kernel<<<grid_for(nE, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(
         nE, d.d1d * d.d1d * d.d1d, op->emask, (double *)op->yE);
      rc = last_launch(ctx, "zero_unmarked");
      if (rc) { return rc; }
   }
   rc = launch_csr_scatter<double>(ctx, d.ndofs, d.offsets, d.indices, (const double *)op->yE,
                                   diag, nullptr, nullptr, false, true);
   if (rc || !op->mask) { return rc; }
   set_mask_one_kernel<<<grid_for(d.ndofs, 256), 256, 0, ctx->stream>>>(d.ndofs, op->mask, diag);
   return last_launch(ctx, "diag_ess_one");
}

// ------------------------------------------------------------------- PCG
static int ensure_pcg_workspace(gbpa_operator *op)
{
   const int64_t n = op->d.ndofs;
   if (op->ws_n >= n && op->state) { return GBPA_SUCCESS; }
   const size_t w = elem_bytes(op->d);
   cudaFree(op->r); cudaFree(op->dv); cudaFree(op->z); cudaFree(op->partials); cudaFree(op->state);
   op->r = op->dv = op->z = nullptr; op->partials = nullptr; op->state = nullptr;
   int rc = check_cuda(cudaMalloc(&op->r, w * n), "cudaMalloc(r)");
   if (!rc) { rc = check_cuda(cudaMalloc(&op->dv, w * n), "cudaMalloc(d)"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&op->z, w * n), "cudaMalloc(z)"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&op->partials, sizeof(double) * 4096), "cudaMalloc(partials)"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&op->state, sizeof(PcgState)), "cudaMalloc(state)"); }
   if (!rc) { rc = check_cuda(cudaMemset(op->state, 0, sizeof(PcgState)), "memset(state)"); }
   if (!rc) { op->ws_n = n; }
   if (op->graph) { cudaGraphExecDestroy(op->graph); op->graph = nullptr; }
   return rc;
}

static int pcg_check_every()
{
   const char *s = getenv("GBPA_PCG_CHECK_EVERY");
   const int k = s ? atoi(s) : 10;
   return k >= 1 && k <= 1000 ? k : 10;
}

// z = A d (constrained: z[ess] = d[ess]), den = (d, z), alpha = nom / den:
// the element apply into the E-vector then the CSR scatter with the dot, or,
// for an operator with the atomic scatter, the apply summing into z (zeroed
// first) then the dot. Both skip their work once the state reports done.
template <typename T>
static int pcg_apply_den(gbpa_operator *op, T *d, T *z, unsigned grid, int first)
{
   gbpa_ctx *ctx = op->ctx;
   const int64_t n = op->d.ndofs;
   int rc;
   if (atomic_scatter(op))
   {
      rc = check_cuda(cudaMemsetAsync(z, 0, sizeof(T) * n, ctx->stream), "memset(z)");
      if (!rc) { rc = apply_to<T>(op, d, z, GBPA_OUT_ATOMIC, &op->state->done); }
      if (rc) { return rc; }
      pcg_scatter_den_kernel<T><<<grid, PCG_BLOCK, 0, ctx->stream>>>(
         op->d.ndofs, nullptr, nullptr, nullptr, z, d, op->mask, op->partials + 2048, op->state, first);
      return last_launch(ctx, "pcg_den");
   }
   rc = apply_evec<T>(op, d, &op->state->done);
   if (rc) { return rc; }
   pcg_scatter_den_kernel<T><<<grid, PCG_BLOCK, 0, ctx->stream>>>(
      op->d.ndofs, op->d.offsets, op->d.indices, (const T *)op->yE, z, d, op->mask,
      op->partials + 2048, op->state, first);
   return last_launch(ctx, "pcg_scatter_den");
}

// One PCG iteration body: update (x, r, z, betanom), direction, A d, den.// One PCG iteration body: update (x, r, z, betanom), direction, A d, den.
template <typename T>
static int pcg_iteration(gbpa_operator *op, T *x, const T *dinv, unsigned grid)
{
   gbpa_ctx *ctx = op->ctx;
   const int64_t n = op->d.ndofs;
   T *r = (T *)op->r, *d = (T *)op->dv, *z = (T *)op->z;
   pcg_update_kernel<T><<<grid, PCG_BLOCK, 0, ctx->stream>>>(n, x, r, z, d, dinv, op->partials,
                                                           op->state);
   int rc = last_launch(ctx, "pcg_update");
   if (rc) { return rc; }
   pcg_direction_kernel<T><<<grid, PCG_BLOCK, 0, ctx->stream>>>(n, z, d, op->state);
   rc = last_launch(ctx, "pcg_direction");
   if (rc) { return rc; }
   return pcg_apply_den<T>(op, d, z, grid, 0);
}

// Runs captured K-iteration graphs of pcg_iteration (x, dinv fixed) until
// the device state reports done, polling the flag between graph launches.
template <typename T>
static int pcg_graph_loop(gbpa_operator *op, T *x, const T *dinv, int max_it)
{
   gbpa_ctx *ctx = op->ctx;
   const int64_t n = op->d.ndofs;
   const unsigned grid = grid_for(n, PCG_BLOCK, 4 * ctx->num_sms);
   int rc = GBPA_SUCCESS;
   const int K = pcg_check_every();
   if (!op->graph || op->graph_x != (const void *)x || op->graph_dinv != (const void *)dinv)
   {
      if (op->graph) { cudaGraphExecDestroy(op->graph); op->graph = nullptr; }
      // Capture on a private non-blocking stream (the context's stream may be
      // the legacy default stream, which cannot be captured); the graph is
      // then launched on the context's stream.
      if (!ctx->capture_stream)
      {
         rc = check_cuda(cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking),
                         "cudaStreamCreate(capture)");
         if (rc) { return rc; }
      }
      cudaGraph_t g = nullptr;
      cudaStream_t saved = ctx->stream;
      const int64_t launches0 = ctx->launches;   // captured launches are counted when they run
      rc = check_cuda(cudaStreamBeginCapture(ctx->capture_stream, cudaStreamCaptureModeThreadLocal),
                      "cudaStreamBeginCapture");
      if (rc) { return rc; }
      ctx->stream = ctx->capture_stream;
      for (int k = 0; k < K && !rc; ++k) { rc = pcg_iteration<T>(op, x, dinv, grid); }
      ctx->stream = saved;
      ctx->launches = launches0;
      const int rc2 = check_cuda(cudaStreamEndCapture(ctx->capture_stream, &g), "cudaStreamEndCapture");
      if (rc || rc2)
      {
         if (g) { cudaGraphDestroy(g); }
         return rc ? rc : rc2;
      }
      rc = check_cuda(cudaGraphInstantiate(&op->graph, g, 0), "cudaGraphInstantiate");
      cudaGraphDestroy(g);
      if (rc) { return rc; }
      op->graph_x = x; op->graph_dinv = dinv;
   }
   int *h_done = (int *)ctx->h_pinned;
   // graph launches are counted as K iterations' worth of kernels
   const int per_iter = 4;
   for (int launched = 0; ; launched += K)
   {
      rc = check_cuda(cudaMemcpyAsync(h_done, &op->state->done, sizeof(int),
                                      cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync(done)");
      if (rc) { return rc; }
      rc = check_cuda(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
      if (rc) { return rc; }
      if (*h_done) { break; }
      if (launched > max_it + K) { break; }   // safety net; the device caps iterations
      rc = check_cuda(cudaGraphLaunch(op->graph, ctx->stream), "cudaGraphLaunch");
      if (rc) { return rc; }
      ctx->launches += (int64_t)K * per_iter;
   }
   return GBPA_SUCCESS;
}

template <typename T>
static int pcg_run(gbpa_operator *op, const T *dinv, const T *b, T *x, double rel_tol,
                   double abs_tol, int max_it, int iterative, gbpa_solve_info *info,
                   float *elapsed_ms)
{
   gbpa_ctx *ctx = op->ctx;
   const int64_t n = op->d.ndofs;
   int rc = ensure_pcg_workspace(op);
   if (rc) { return rc; }
   T *r = (T *)op->r, *d = (T *)op->dv, *z = (T *)op->z;
   // 4 blocks of 512 threads per SM: full occupancy for the streaming vector
   // phases (partials buffer holds 2048 entries per reduction)
   const unsigned grid = grid_for(n, PCG_BLOCK, 4 * ctx->num_sms);
   StreamTimer timer(ctx->stream);
   PcgState h{};
   h.rel_tol2 = rel_tol * rel_tol;
   h.abs_tol2 = abs_tol * abs_tol;
   h.max_it = max_it;
   rc = check_cuda(cudaMemcpyAsync(op->state, &h, sizeof(PcgState), cudaMemcpyHostToDevice,
                                   ctx->stream), "cudaMemcpyAsync(state)");
   if (rc) { return rc; }
   if (iterative)
   {
      rc = op_mult<T>(op, x, r);   // r = A x, then r = b - r in the init kernel
      if (rc) { return rc; }
   }
   pcg_init_kernel<T><<<grid, PCG_BLOCK, 0, ctx->stream>>>(n, b, x, r, z, d, dinv, iterative,
                                                         op->partials, op->state);
   rc = last_launch(ctx, "pcg_init");
   if (rc) { return rc; }
   // z = A d, den = (d, z), alpha = nom / den
   rc = pcg_apply_den<T>(op, d, z, grid, 1);
   if (rc) { return rc; }

   rc = pcg_graph_loop<T>(op, x, dinv, max_it);
   if (rc) { return rc; }
   const float ms = timer.stop(ctx->stream);
   if (elapsed_ms) { *elapsed_ms = ms; }
   rc = check_cuda(cudaMemcpy(&h, op->state, sizeof(PcgState), cudaMemcpyDeviceToHost),
                   "cudaMemcpy(state)");
   if (rc) { return rc; }
   if (info)
   {
      info->iterations = h.final_iter;
      info->converged = h.converged;
      info->initial_norm = h.nom0 >= 0 ? sqrt(h.nom0) : h.nom0;
      info->final_norm = h.betanom >= 0 ? sqrt(h.betanom) : h.betanom;
   }
   if (h.status) { return h.status; }
   return GBPA_SUCCESS;
}

// ||b - A x|| / ||b|| in FP64 (op must be FP64); uses op->r64/t64.
static int true_residual(gbpa_operator *op, const double *b, const double *x, double *rel)
{
   gbpa_ctx *ctx = op->ctx;
   const int64_t n = op->d.ndofs;
   if (!op->r64)
   {
      int rc = check_cuda(cudaMalloc(&op->r64, sizeof(double) * n), "cudaMalloc(r64)");
      if (!rc) { rc = check_cuda(cudaMalloc(&op->t64, sizeof(double) * 8), "cudaMalloc(t64)"); }
      if (rc) { return rc; }
   }
   int rc = op_mult<double>(op, x, op->r64);
   if (rc) { return rc; }
   residual_kernel<<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(n, b, op->r64);
   rc = last_launch(ctx, "residual");
   if (rc) { return rc; }
   rc = launch_dot<double>(ctx, n, op->r64, op->r64, op->t64);
   if (!rc) { rc = launch_dot<double>(ctx, n, b, b, op->t64 + 1); }
   if (rc) { return rc; }
   double h[2];
   rc = check_cuda(cudaMemcpyAsync(h, op->t64, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                   ctx->stream), "cudaMemcpyAsync");
   if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
   *rel = h[1] > 0 ? sqrt(h[0] / h[1]) : sqrt(h[0]);
   return rc;
}

extern "C" int gbpa_pcg_solve(gbpa_operator_t A, const double *dinv, const double *b, double *x,
                              double rel_tol, double abs_tol, int max_it, int iterative_mode,
                              gbpa_solve_info *info)
{
   if (!A || (A->d.ndofs > 0 && (!dinv || !b || !x)) || max_it < 0 || rel_tol < 0 || abs_tol < 0)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (A->d.precision == GBPA_F32) { return GBPA_ERR_INVALID_ARGUMENT; }
   gbpa_solve_info tmp{};
   gbpa_solve_info *inf = info ? info : &tmp;
   memset(inf, 0, sizeof(*inf));
   if (A->d.ndofs == 0) { inf->converged = 1; return GBPA_SUCCESS; }
   float ms = 0.f;
   int rc = pcg_run<double>(A, dinv, b, x, rel_tol, abs_tol, max_it, iterative_mode, inf, &ms);
   inf->seconds = ms * 1e-3;
   if (rc) { return rc; }
   inf->outer_iterations = 1;
   inf->inner_iterations = inf->iterations;
   return true_residual(A, b, x, &inf->true_rel_residual);
}

// FP32 Jacobi-PCG on an FP32 operator (zero initial guess), for callers
// inside the library (the multigrid coarse solve in FP32).
int gbpa::pcg_solve_f32(gbpa_operator *A, const float *dinv, const float *b, float *x, double rel_tol,
                        double abs_tol, int max_it, gbpa_solve_info *info)
{
   memset(info, 0, sizeof(*info));
   if (A->d.ndofs == 0) { info->converged = 1; return GBPA_SUCCESS; }
   return pcg_run<float>(A, dinv, b, x, rel_tol, abs_tol, max_it, 0, info, nullptr);
}

extern "C" int gbpa_pcg_solve_mixed(gbpa_operator_t A64, gbpa_operator_t A32, const float *dinv32,
                                    const double *b, double *x, double outer_rel_tol,
                                    double inner_rel_tol, int max_outer, int max_inner,
                                    gbpa_solve_info *info)
{
   if (!A64 || !A32 || A64->d.precision == GBPA_F32 || A32->d.precision != GBPA_F32 ||
       A64->d.ndofs != A32->d.ndofs || A64->ctx != A32->ctx || max_outer < 1 || max_inner < 1)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   const int64_t n = A64->d.ndofs;
   if (n > 0 && (!dinv32 || !b || !x)) { return GBPA_ERR_INVALID_ARGUMENT; }
   gbpa_solve_info tmp{};
   gbpa_solve_info *inf = info ? info : &tmp;
   memset(inf, 0, sizeof(*inf));
   if (n == 0) { inf->converged = 1; return GBPA_SUCCESS; }
   gbpa_ctx *ctx = A64->ctx;
   int rc = ensure_pcg_workspace(A32);
   if (rc) { return rc; }
   if (!A64->r64)
   {
      rc = check_cuda(cudaMalloc(&A64->r64, sizeof(double) * n), "cudaMalloc(r64)");
      if (!rc) { rc = check_cuda(cudaMalloc(&A64->t64, sizeof(double) * 8), "cudaMalloc(t64)"); }
      if (rc) { return rc; }
   }
   // inner-solve vectors: rhs and correction in FP32 (separate from A32's PCG workspace)
   float *r32 = (float *)scratch(ctx, SLOT_PCG32, sizeof(float) * 2 * n);
   if (!r32) { return GBPA_ERR_OUT_OF_MEMORY; }
   float *c32 = r32 + n;
   StreamTimer timer(ctx->stream);
   // x = 0, r = b
   rc = check_cuda(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream), "memset(x)");
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(A64->r64, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream), "copy"); }
   if (!rc) { rc = launch_dot<double>(ctx, n, b, b, A64->t64 + 1); }
   if (rc) { return rc; }
   double hb[2];
   int outer = 0, inner_total = 0, converged = 0;
   double rel = 1.0;
   for (outer = 0; outer <= max_outer; ++outer)
   {
      rc = launch_dot<double>(ctx, n, A64->r64, A64->r64, A64->t64);
      if (rc) { return rc; }
      rc = check_cuda(cudaMemcpyAsync(hb, A64->t64, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                      ctx->stream), "cudaMemcpyAsync");
      if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
      if (rc) { return rc; }
      rel = hb[1] > 0 ? sqrt(hb[0] / hb[1]) : sqrt(hb[0]);
      if (!std::isfinite(rel)) { return GBPA_ERR_NOT_FINITE; }
      if (rel <= outer_rel_tol) { converged = 1; break; }
      if (outer == max_outer || hb[0] == 0.0) { break; }
      // r32 = r / ||r||; solve A32 c = r32 to inner_rel_tol; x += ||r|| c
      scale_to_f32_kernel<<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(
         n, A64->r64, A64->t64, r32);
      rc = last_launch(ctx, "scale_to_f32");
      if (rc) { return rc; }
      gbpa_solve_info ii{};
      rc = pcg_run<float>(A32, dinv32, r32, c32, inner_rel_tol, 0.0, max_inner, 0, &ii, nullptr);
      if (rc) { return rc; }
      inner_total += ii.iterations;
      correct_kernel<<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(n, x, c32,
                                                                                A64->t64);
      rc = last_launch(ctx, "correct");
      if (rc) { return rc; }
      // true residual in FP64: r = b - A64 x
      rc = op_mult<double>(A64, x, A64->r64);
      if (rc) { return rc; }
      residual_kernel<<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(n, b, A64->r64);
      rc = last_launch(ctx, "residual");
      if (rc) { return rc; }
   }
   const float ms = timer.stop(ctx->stream);
   inf->seconds = ms * 1e-3;
   inf->outer_iterations = outer;
   inf->inner_iterations = inner_total;
   inf->iterations = inner_total;
   inf->converged = converged;
   inf->true_rel_residual = rel;
   inf->final_norm = sqrt(hb[0]);
   return converged ? GBPA_SUCCESS : GBPA_ERR_NOT_CONVERGED;
}

// Mixed precision with reliable updates: ONE FP32 Jacobi-PCG on A32 whose
// iterated residual is replaced by the true FP64 residual b - A64 x each time
// it has dropped by delta since the last replacement, the search direction
// keeping its history (residual replacement: Sleijpen and van der Vorst 1996;
// van der Vorst and Ye 2000). Unlike restarted defect correction the Krylov
// space is never discarded, so the FP32 iteration count stays close to the
// FP64 one. The FP32 vectors carry the problem scaled by 1/||b||; x and the
// true residual stay FP64; stop when ||b - A64 x|| <= rel_tol ||b||.
extern "C" int gbpa_pcg_solve_mixed_reliable(gbpa_operator_t A64, gbpa_operator_t A32,
                                             const float *dinv32, const double *b, double *x,
                                             double rel_tol, double delta, int max_it,
                                             gbpa_solve_info *info)
{
   if (!A64 || !A32 || A64->d.precision == GBPA_F32 || A32->d.precision != GBPA_F32 ||
       A64->d.ndofs != A32->d.ndofs || A64->ctx != A32->ctx || max_it < 1 || rel_tol < 0 ||
       !(delta > 0.0 && delta < 1.0))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   const int64_t n = A64->d.ndofs;
   if (n > 0 && (!dinv32 || !b || !x)) { return GBPA_ERR_INVALID_ARGUMENT; }
   gbpa_solve_info tmp{};
   gbpa_solve_info *inf = info ? info : &tmp;
   memset(inf, 0, sizeof(*inf));
   if (n == 0) { inf->converged = 1; return GBPA_SUCCESS; }
   gbpa_ctx *ctx = A64->ctx;
   gbpa_operator *op = A32;
   int rc = ensure_pcg_workspace(op);
   if (rc) { return rc; }
   if (!A64->r64)
   {
      rc = check_cuda(cudaMalloc(&A64->r64, sizeof(double) * n), "cudaMalloc(r64)");
      if (!rc) { rc = check_cuda(cudaMalloc(&A64->t64, sizeof(double) * 8), "cudaMalloc(t64)"); }
      if (rc) { return rc; }
   }
   // FP32 correction since the last update (x32) and the scaled right-hand side (b32)
   float *x32 = (float *)scratch(ctx, SLOT_PCG32, sizeof(float) * 2 * n);
   if (!x32) { return GBPA_ERR_OUT_OF_MEMORY; }
   float *b32 = x32 + n;
   float *r = (float *)op->r, *d = (float *)op->dv, *z = (float *)op->z;
   const unsigned grid = grid_for(n, PCG_BLOCK, 4 * ctx->num_sms);
   const unsigned vg = grid_for(n, 256, 8 * ctx->num_sms);
   StreamTimer timer(ctx->stream);
   double hb[2] = {0.0, 0.0};
   double rel = 1.0;
   int updates = 0, converged = 0;
   PcgState h{};
   // x = 0; t64[1] = (b, b); b32 = b / ||b||
   rc = check_cuda(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream), "memset(x)");
   if (!rc) { rc = launch_dot<double>(ctx, n, b, b, A64->t64 + 1); }
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(hb + 1, A64->t64 + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "copy"); }
   if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
   if (rc) { return rc; }
   if (!std::isfinite(hb[1])) { return GBPA_ERR_NOT_FINITE; }
   if (hb[1] == 0.0)
   {
      inf->converged = 1;
      return GBPA_SUCCESS;
   }
   scale_to_f32_kernel<<<vg, 256, 0, ctx->stream>>>(n, b, A64->t64 + 1, b32);
   rc = last_launch(ctx, "scale_to_f32");
   if (rc) { return rc; }
   // FP32 CG start: x32 = 0, r = b32, z = dinv r, d = z, segment ends at delta^2 (r, z)
   h.rel_tol2 = delta * delta;
   h.max_it = max_it;
   rc = check_cuda(cudaMemcpyAsync(op->state, &h, sizeof(PcgState), cudaMemcpyHostToDevice,
                                   ctx->stream), "cudaMemcpyAsync(state)");
   if (rc) { return rc; }
   pcg_init_kernel<float><<<grid, PCG_BLOCK, 0, ctx->stream>>>(n, b32, x32, r, z, d, dinv32, 0,
                                                              op->partials, op->state);
   rc = last_launch(ctx, "pcg_init");
   if (!rc) { rc = pcg_apply_den<float>(op, d, z, grid, 1); }
   if (rc) { return rc; }
   for (;;)
   {
      // FP32 iterations of this segment
      rc = pcg_graph_loop<float>(op, x32, dinv32, max_it);
      if (rc) { return rc; }
      rc = check_cuda(cudaMemcpyAsync(&h, op->state, sizeof(PcgState), cudaMemcpyDeviceToHost,
                                      ctx->stream), "copy(state)");
      if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
      if (rc) { return rc; }
      if (h.status) { return h.status; }
      // reliable update: x += ||b|| x32, x32 = 0, r64 = b - A64 x (FP64)
      correct_kernel<<<vg, 256, 0, ctx->stream>>>(n, x, x32, A64->t64 + 1);
      rc = last_launch(ctx, "correct");
      if (!rc) { rc = check_cuda(cudaMemsetAsync(x32, 0, sizeof(float) * n, ctx->stream), "memset"); }
      if (!rc) { rc = op_mult<double>(A64, x, A64->r64); }
      if (!rc)
      {
         residual_kernel<<<vg, 256, 0, ctx->stream>>>(n, b, A64->r64);
         rc = last_launch(ctx, "residual");
      }
      if (!rc) { rc = launch_dot<double>(ctx, n, A64->r64, A64->r64, A64->t64); }
      if (!rc) { rc = check_cuda(cudaMemcpyAsync(hb, A64->t64, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "copy"); }
      if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
      if (rc) { return rc; }
      ++updates;
      rel = sqrt(hb[0] / hb[1]);
      if (!std::isfinite(rel)) { return GBPA_ERR_NOT_FINITE; }
      if (rel <= rel_tol) { converged = 1; break; }
      if (h.iter > max_it || (h.done && !h.converged)) { break; }   // iteration cap or breakdown
      // r = r64 / ||b|| in FP32; z = dinv r; beta; the direction continues
      scale_to_f32_kernel<<<vg, 256, 0, ctx->stream>>>(n, A64->r64, A64->t64 + 1, r);
      rc = last_launch(ctx, "scale_to_f32");
      if (!rc)
      {
         pcg_restart_kernel<<<grid, PCG_BLOCK, 0, ctx->stream>>>(n, r, z, dinv32, op->partials, op->state);
         rc = last_launch(ctx, "pcg_restart");
      }
      if (!rc)
      {
         pcg_direction_kernel<float><<<grid, PCG_BLOCK, 0, ctx->stream>>>(n, z, d, op->state);
         rc = last_launch(ctx, "pcg_direction");
      }
      if (!rc) { rc = pcg_apply_den<float>(op, d, z, grid, 0); }
      if (rc) { return rc; }
   }
   const float ms = timer.stop(ctx->stream);
   inf->seconds = ms * 1e-3;
   inf->outer_iterations = updates;
   inf->inner_iterations = h.iter;
   inf->iterations = h.iter;
   inf->converged = converged;
   inf->true_rel_residual = rel;
   inf->initial_norm = sqrt(hb[1]);
   inf->final_norm = sqrt(hb[0]);
   return converged ? GBPA_SUCCESS : GBPA_ERR_NOT_CONVERGED;
}
