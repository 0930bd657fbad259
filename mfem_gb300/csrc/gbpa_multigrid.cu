// p-multigrid around the PA diffusion operator (the structure of the
// reference's examples/ex26.cpp):
//   transfer     TensorProductPRefinementTransferOperator
//                (fem/transfer.cpp:2620-2990): prolongation
//                y_f = R_f^T (mask .* I (R_c x_c)), restriction its transpose;
//                mask = ElementRestriction::BooleanMask (fem/restriction.cpp:
//                255-292), 1 on the first slot of each fine dof's CSR row
//   smoother     OperatorChebyshevSmoother (linalg/solvers.cpp:455-660) with
//                the PowerMethod eigenvalue estimate (linalg/operator.cpp:
//                886-942)
//   cycle        MultigridBase::Cycle, V(1,1) (fem/multigrid.cpp:106-239),
//                level 0 solved by CG to a relative tolerance
//   outer solve  CGSolver::Mult (linalg/solvers.cpp:869-1050) preconditioned
//                by the V-cycle
// Levels are operators with FP64 vectors (GBPA_F64, GBPA_F64X2) or all with
// FP32 vectors (GBPA_F32: the V-cycle then preconditions the FP64 CG in FP32).
//
// GPU layout. The prolongation writes every fine dof exactly once, from its
// mask-owning element slot (no scatter, no atomics); the restriction writes
// a coarse E-vector and sums it with the deterministic CSR scatter. Both are
// three tensor contractions per element in a (Df, Df, nbz) block with the
// element's values in shared memory.
#include "gbpa_csr.cuh"
#include "gbpa_operator.cuh"
#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

namespace gbpa
{
constexpr int MG_MAX_1D = 10;   // largest D1D of a transfer level (p <= 9)

// Fine slot owners: own[s] = 1 on the first slot of each fine dof's CSR row.
__global__ void mg_owner_kernel(int ndofs, const int *__restrict__ offsets, const int *__restrict__ indices,
                                unsigned char *__restrict__ own)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndofs; i += gridDim.x * blockDim.x)
   {
      const int j0 = offsets[i], j1 = offsets[i + 1];
      for (int j = j0; j < j1; ++j)
      {
         const int s = indices[j];
         own[s >= 0 ? s : -1 - s] = j == j0 ? 1 : 0;
      }
   }
}

// Prolongation: one element per z-slice of the block, threads (qx, qy).
// Bi (df, dc) column-major: Bi[q + df * d].
template <typename T>
__global__ void mg_prolong_kernel(int ne, int dc, int df, const T *__restrict__ Bi,
                                  const int *__restrict__ gm_c, const int *__restrict__ gm_f,
                                  const unsigned char *__restrict__ own, const T *__restrict__ xc,
                                  T *__restrict__ yf)
{
   extern __shared__ __align__(16) unsigned char sm_raw[];
   T *sm = reinterpret_cast<T *>(sm_raw);
   const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
   const int e = blockIdx.x * blockDim.z + tz;
   const int dc3 = dc * dc * dc, nthr = df * df * blockDim.z, tid = tx + df * (ty + df * tz);
   T *sB = sm;                                          // [df][dc]
   const int per = dc3 + dc * dc * df + dc * df * df;   // X | T1 | T2
   T *X = sm + df * dc + tz * per;
   T *T1 = X + dc3, *T2 = T1 + dc * dc * df;
   for (int i = tid; i < df * dc; i += nthr) { sB[i] = Bi[i]; }
   const bool active = e < ne;
   if (active)
   {
      for (int i = tx + df * ty; i < dc3; i += df * df)
      {
         const int g = gm_c[(long long)e * dc3 + i];
         const T v = xc[g >= 0 ? g : -1 - g];
         X[i] = g >= 0 ? v : -v;
      }
   }
   __syncthreads();
   // x: T1[dz][dy][qx] = sum_dx B(qx, dx) X[dz][dy][dx]   (thread (qx, dy))
   if (active && ty < dc)
   {
      for (int dz = 0; dz < dc; ++dz)
      {
         T s = T(0);
         for (int dx = 0; dx < dc; ++dx) { s += sB[tx + df * dx] * X[dx + dc * (ty + dc * dz)]; }
         T1[tx + df * (ty + dc * dz)] = s;
      }
   }
   __syncthreads();
   // y: T2[dz][qy][qx] = sum_dy B(qy, dy) T1[dz][dy][qx]   (thread (qx, qy))
   if (active)
   {
      for (int dz = 0; dz < dc; ++dz)
      {
         T s = T(0);
         for (int dy = 0; dy < dc; ++dy) { s += sB[ty + df * dy] * T1[tx + df * (dy + dc * dz)]; }
         T2[tx + df * (ty + df * dz)] = s;
      }
   }
   __syncthreads();
   // z: Y[qz][qy][qx] = sum_dz B(qz, dz) T2[dz][qy][qx]; the owning slot
   // writes its fine dof
   if (active)
   {
      const int df3 = df * df * df;
      for (int qz = 0; qz < df; ++qz)
      {
         T s = T(0);
         for (int dz = 0; dz < dc; ++dz) { s += sB[qz + df * dz] * T2[tx + df * (ty + df * dz)]; }
         const long long slot = (long long)e * df3 + tx + df * (ty + df * qz);
         if (own[slot])
         {
            const int g = gm_f[slot];
            if (g >= 0) { yf[g] = s; } else { yf[-1 - g] = -s; }
         }
      }
   }
}

// Restriction (the transpose) into a coarse E-vector: X = mask .* R_f x_f,
// then the transposed contractions; threads (qx, qy) of the fine slab.
template <typename T>
__global__ void mg_restrict_kernel(int ne, int dc, int df, const T *__restrict__ Bi,
                                   const int *__restrict__ gm_f, const unsigned char *__restrict__ own,
                                   const T *__restrict__ xf, T *__restrict__ yEc)
{
   extern __shared__ __align__(16) unsigned char sm_raw[];
   T *sm = reinterpret_cast<T *>(sm_raw);
   const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
   const int e = blockIdx.x * blockDim.z + tz;
   const int df3 = df * df * df, dc3 = dc * dc * dc, nthr = df * df * blockDim.z;
   const int tid = tx + df * (ty + df * tz);
   T *sB = sm;
   const int per = df3 + df * df * dc + df * dc * dc;   // X | T1 | T2
   T *X = sm + df * dc + tz * per;
   T *T1 = X + df3, *T2 = T1 + df * df * dc;
   for (int i = tid; i < df * dc; i += nthr) { sB[i] = Bi[i]; }
   const bool active = e < ne;
   if (active)
   {
      for (int i = tx + df * ty; i < df3; i += df * df)
      {
         const long long slot = (long long)e * df3 + i;
         T v = T(0);
         if (own[slot])
         {
            const int g = gm_f[slot];
            const T a = xf[g >= 0 ? g : -1 - g];
            v = g >= 0 ? a : -a;
         }
         X[i] = v;
      }
   }
   __syncthreads();
   // x: T1[qz][qy][dx] = sum_qx B(qx, dx) X[qz][qy][qx]   (thread (dx, qy))
   if (active && tx < dc)
   {
      for (int qz = 0; qz < df; ++qz)
      {
         T s = T(0);
         for (int qx = 0; qx < df; ++qx) { s += sB[qx + df * tx] * X[qx + df * (ty + df * qz)]; }
         T1[tx + dc * (ty + df * qz)] = s;
      }
   }
   __syncthreads();
   // y: T2[qz][dy][dx] = sum_qy B(qy, dy) T1[qz][qy][dx]   (thread (dx, dy))
   if (active && tx < dc && ty < dc)
   {
      for (int qz = 0; qz < df; ++qz)
      {
         T s = T(0);
         for (int qy = 0; qy < df; ++qy) { s += sB[qy + df * ty] * T1[tx + dc * (qy + df * qz)]; }
         T2[tx + dc * (ty + dc * qz)] = s;
      }
   }
   __syncthreads();
   // z: Y[dz][dy][dx] = sum_qz B(qz, dz) T2[qz][dy][dx]
   if (active && tx < dc && ty < dc)
   {
      for (int dz = 0; dz < dc; ++dz)
      {
         T s = T(0);
         for (int qz = 0; qz < df; ++qz) { s += sB[qz + df * dz] * T2[tx + dc * (ty + dc * qz)]; }
         yEc[(long long)e * dc3 + tx + dc * (ty + dc * dz)] = s;
      }
   }
}

// ---- vector kernels of the smoother, the cycle and the outer CG
template <typename T>
__global__ void mg_scale_kernel(int64_t n, const T *__restrict__ d, const T *__restrict__ x,
                                T *__restrict__ r, T *__restrict__ y, T c, int first)
{
   // r = d .* x; y = c r (first) or y += c r
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
   {
      const T v = d[i] * x[i];
      r[i] = v;
      y[i] = first ? c * v : y[i] + c * v;
   }
}
template <typename T>
__global__ void mg_mul_kernel(int64_t n, const T *__restrict__ d, T *__restrict__ y)
{
   // y .*= d
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
   {
      y[i] *= d[i];
   }
}
template <typename T>
__global__ void mg_axpby_kernel(int64_t n, T a, const T *x, T b, T *y)
{
   // y = a x + b y (x may alias y)
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
   {
      y[i] = a * x[i] + b * y[i];
   }
}
template <typename T>
__global__ void mg_fill_kernel(int64_t n, T v, T *__restrict__ y)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
   {
      y[i] = v;
   }
}
// splitmix64 at counter i of the stream seeded with `seed`, in [0, 1)
template <typename T>
__global__ void mg_random_kernel(int64_t n, unsigned long long seed, T *__restrict__ y)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
   {
      unsigned long long z = seed + (unsigned long long)(i + 1) * 0x9e3779b97f4a7c15ULL;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
      z ^= z >> 31;
      y[i] = (T)((double)(z >> 11) * (1.0 / 9007199254740992.0));
   }
}
template <typename T>
__global__ void mg_dinv_kernel(int n, const double *__restrict__ diag, T *__restrict__ dinv)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
   {
      dinv[i] = (T)(1.0 / diag[i]);
   }
}
template <typename T>
__global__ void mg_convert_kernel(int64_t n, const double *__restrict__ x, T *__restrict__ y)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
   {
      y[i] = (T)x[i];
   }
}
template <typename T>
__global__ void mg_widen_kernel(int64_t n, const T *__restrict__ x, double *__restrict__ y)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
   {
      y[i] = (double)x[i];
   }
}
template <typename T>
__global__ void mg_set_ess_kernel(int n_ess, const int *__restrict__ ess, T v, T *__restrict__ y)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_ess; i += gridDim.x * blockDim.x)
   {
      y[ess[i]] = v;
   }
}

static unsigned vgrid(gbpa_ctx *ctx, int64_t n) { return grid_for(n, 256, 8 * ctx->num_sms); }

} // namespace gbpa

using namespace gbpa;

// ------------------------------------------------------------------ objects
struct gbpa_ptransfer
{
   gbpa_ctx *ctx = nullptr;
   int ne = 0, dc = 0, df = 0, ndofs_c = 0, ndofs_f = 0;
   bool f32 = false;                // vectors in float (GBPA_F32) or double
   const int *gm_c = nullptr, *off_c = nullptr, *ind_c = nullptr, *gm_f = nullptr;
   void *Bi = nullptr;              // device copy (df, dc) in the vector type
   unsigned char *own = nullptr;    // fine slot owners
   void *yEc = nullptr;             // coarse E-vector scratch
};

struct gbpa_chebyshev
{
   gbpa_operator *A = nullptr;
   bool f32 = false;
   int order = 0;
   double lambda = 0.0;
   double coeffs[16] = {0};
   void *dinv = nullptr, *res = nullptr, *h = nullptr;
};

struct gbpa_multigrid
{
   gbpa_ctx *ctx = nullptr;
   int nl = 0;
   bool f32 = false;
   std::vector<gbpa_operator *> ops;
   std::vector<gbpa_chebyshev *> sm;
   std::vector<gbpa_ptransfer *> P;
   double coarse_tol = 1e-2;
   int coarse_max = 200;
   void *coarse_dinv = nullptr;        // level-0 CG preconditioner: ones (plain CG) or Jacobi
   std::vector<void *> X, Y, R, Z;     // per level, in the levels' vector type
   double *d_dot = nullptr;
   int64_t coarse_iterations = 0;
};

namespace
{
bool fp32_vectors(const gbpa_operator *A) { return A->d.precision == GBPA_F32; }
size_t vbytes(bool f32) { return f32 ? sizeof(float) : sizeof(double); }
int transfer_nbz(int df) { return std::max(1, 128 / (df * df)); }
int dev_alloc(void **p, size_t bytes) { return check_cuda(cudaMalloc(p, bytes > 0 ? bytes : 16), "cudaMalloc"); }

// Chebyshev coefficients: 1 - t p(t) = T_k((theta - t)/delta) / T_k(theta/delta)
// on [0.3, 1.2] * lambda (linalg/solvers.cpp:552-616 lists the closed forms
// for orders 1-5). The Chebyshev recurrence T_{m+1} = 2 s T_m - T_{m-1} is
// expanded at s = (theta - t)/delta as polynomials in t; c_{j-1} = -e_j/e_0.
void chebyshev_coeffs(int order, double lambda, double *c)
{
   const double up = 1.2 * lambda, lo = 0.3 * lambda;
   const double theta = 0.5 * (up + lo), delta = 0.5 * (up - lo);
   const double a = theta / delta, b = -1.0 / delta;
   double Pm[16] = {0}, P[16] = {0}, Pn[16];
   Pm[0] = 1.0;
   P[0] = a; P[1] = b;
   for (int m = 1; m < order; ++m)
   {
      for (int j = 0; j <= m + 1; ++j)
      {
         double v = 2.0 * a * P[j] - Pm[j];
         if (j > 0) { v += 2.0 * b * P[j - 1]; }
         Pn[j] = v;
      }
      for (int j = m + 2; j < 16; ++j) { Pn[j] = 0.0; }
      std::copy(P, P + 16, Pm);
      std::copy(Pn, Pn + 16, P);
   }
   for (int j = 1; j <= order; ++j) { c[j - 1] = -P[j] / P[0]; }
}

template <typename T>
int host_dot(gbpa_ctx *ctx, int64_t n, const T *x, const T *y, double *d_out, double *out)
{
   int rc = launch_dot<T>(ctx, n, x, y, d_out);
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(ctx->h_pinned, d_out, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "copy"); }
   if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
   if (!rc) { *out = ctx->h_pinned[0]; }
   return rc;
}
template <typename T>
int axpby(gbpa_ctx *ctx, int64_t n, double a, const T *x, double b, T *y)
{
   if (n <= 0) { return GBPA_SUCCESS; }
   mg_axpby_kernel<T><<<vgrid(ctx, n), 256, 0, ctx->stream>>>(n, (T)a, x, (T)b, y);
   return last_launch(ctx, "mg_axpby");
}
template <typename T>
int fill(gbpa_ctx *ctx, int64_t n, double v, T *y)
{
   if (n <= 0) { return GBPA_SUCCESS; }
   mg_fill_kernel<T><<<vgrid(ctx, n), 256, 0, ctx->stream>>>(n, (T)v, y);
   return last_launch(ctx, "mg_fill");
}

// ---- transfer
template <typename T>
int ptransfer_mult(gbpa_ptransfer *Tr, const T *xc, T *yf)
{
   const int nbz = transfer_nbz(Tr->df);
   int ne = Tr->ne, dc = Tr->dc, df = Tr->df;
   const size_t smem = sizeof(T) * ((size_t)df * dc + (size_t)nbz * (dc * dc * dc + dc * dc * df + dc * df * df));
   const T *Bi = (const T *)Tr->Bi;
   const int *gc = Tr->gm_c, *gf = Tr->gm_f;
   const unsigned char *own = Tr->own;
   void *args[] = {&ne, &dc, &df, (void *)&Bi, (void *)&gc, (void *)&gf, (void *)&own, (void *)&xc, &yf};
   return launch_generic(Tr->ctx, (const void *)mg_prolong_kernel<T>, dim3((ne + nbz - 1) / nbz), dim3(df, df, nbz),
                         args, smem, "mg_prolong");
}
template <typename T>
int ptransfer_mult_transpose(gbpa_ptransfer *Tr, const T *xf, T *yc)
{
   if (Tr->ne == 0) { return fill<T>(Tr->ctx, Tr->ndofs_c, 0.0, yc); }
   const int nbz = transfer_nbz(Tr->df);
   int ne = Tr->ne, dc = Tr->dc, df = Tr->df;
   const size_t smem = sizeof(T) * ((size_t)df * dc + (size_t)nbz * (df * df * df + df * df * dc + df * dc * dc));
   const T *Bi = (const T *)Tr->Bi;
   const int *gf = Tr->gm_f;
   const unsigned char *own = Tr->own;
   T *yEc = (T *)Tr->yEc;
   void *args[] = {&ne, &dc, &df, (void *)&Bi, (void *)&gf, (void *)&own, (void *)&xf, &yEc};
   int rc = launch_generic(Tr->ctx, (const void *)mg_restrict_kernel<T>, dim3((ne + nbz - 1) / nbz),
                           dim3(df, df, nbz), args, smem, "mg_restrict");
   if (rc) { return rc; }
   return launch_csr_scatter<T>(Tr->ctx, Tr->ndofs_c, Tr->off_c, Tr->ind_c, yEc, yc, nullptr, nullptr, false, false);
}

// ---- Chebyshev: OperatorChebyshevSmoother::Mult (linalg/solvers.cpp:619-656):
// res = x; y = 0; for k: (k > 0: res = A res) res .*= dinv; y += c_k res
template <typename T>
int chebyshev_mult(gbpa_chebyshev *S, const T *x, T *y)
{
   gbpa_ctx *ctx = S->A->ctx;
   const int64_t n = S->A->d.ndofs;
   if (n == 0) { return GBPA_SUCCESS; }
   T *dinv = (T *)S->dinv, *res = (T *)S->res, *h = (T *)S->h;
   int rc = GBPA_SUCCESS;
   for (int k = 0; k < S->order && !rc; ++k)
   {
      const T *src = x;
      if (k > 0)
      {
         rc = gbpa_operator_mult(S->A, res, h);
         src = h;
      }
      if (rc) { break; }
      mg_scale_kernel<T><<<vgrid(ctx, n), 256, 0, ctx->stream>>>(n, dinv, src, res, y, (T)S->coeffs[k], k == 0);
      rc = last_launch(ctx, "mg_scale");
   }
   return rc;
}

// PowerMethod::EstimateLargestEigenvalue (linalg/operator.cpp:886-942) on
// D^-1 A: v0 random, normalised each step, lambda = (v0, D^-1 A v0)
template <typename T>
int power_method(gbpa_chebyshev *S, int steps, double tol, unsigned long long seed, double *out)
{
   gbpa_operator *A = S->A;
   gbpa_ctx *ctx = A->ctx;
   const int64_t n = A->d.ndofs;
   T *v0 = (T *)S->res, *v1 = (T *)S->h;
   double *d_s = nullptr;
   int rc = dev_alloc((void **)&d_s, sizeof(double));
   if (!rc && n > 0)
   {
      mg_random_kernel<T><<<vgrid(ctx, n), 256, 0, ctx->stream>>>(n, seed, v0);
      rc = last_launch(ctx, "mg_random");
   }
   double lam = 1.0;
   for (int it = 0; it < steps && !rc; ++it)
   {
      double nrm2 = 0.0, ln = 0.0;
      rc = host_dot<T>(ctx, n, v0, v0, d_s, &nrm2);
      if (!rc) { rc = axpby<T>(ctx, n, 0.0, v0, 1.0 / std::sqrt(nrm2), v0); }
      if (!rc) { rc = gbpa_operator_mult(A, v0, v1); }
      if (!rc)
      {
         mg_mul_kernel<T><<<vgrid(ctx, n), 256, 0, ctx->stream>>>(n, (const T *)S->dinv, v1);
         rc = last_launch(ctx, "mg_mul");
      }
      if (!rc) { rc = host_dot<T>(ctx, n, v0, v1, d_s, &ln); }
      if (rc) { break; }
      const double diff = std::fabs((ln - lam) / lam);
      lam = ln;
      std::swap(v0, v1);
      if (diff < tol) { break; }
   }
   cudaFree(d_s);
   *out = lam;
   return rc;
}

template <typename T>
int coarse_solve(gbpa_multigrid *M, gbpa_solve_info *info);
template <>
int coarse_solve<double>(gbpa_multigrid *M, gbpa_solve_info *info)
{
   return gbpa_pcg_solve(M->ops[0], (const double *)M->coarse_dinv, (const double *)M->X[0], (double *)M->Y[0],
                         M->coarse_tol, 0.0, M->coarse_max, 0, info);
}
template <>
int coarse_solve<float>(gbpa_multigrid *M, gbpa_solve_info *info)
{
   return pcg_solve_f32(M->ops[0], (const float *)M->coarse_dinv, (const float *)M->X[0], (float *)M->Y[0],
                        M->coarse_tol, 0.0, M->coarse_max, info);
}

// MultigridBase::Cycle (fem/multigrid.cpp:179-239), V(1,1); X[level] holds
// the right-hand side, Y[level] receives the correction.
template <typename T>
int mg_cycle(gbpa_multigrid *M, int level)
{
   gbpa_ctx *ctx = M->ctx;
   gbpa_operator *A = M->ops[level];
   const int64_t n = A->d.ndofs;
   T *X = (T *)M->X[level], *Y = (T *)M->Y[level], *R = (T *)M->R[level], *Z = (T *)M->Z[level];
   if (level == 0)
   {
      // CGSolver to the coarse tolerance: without preconditioner (plain CG is
      // Jacobi-PCG with a unit inverse diagonal) or with Jacobi
      gbpa_solve_info info;
      const int rc = coarse_solve<T>(M, &info);
      M->coarse_iterations += info.iterations;
      return rc == GBPA_ERR_NOT_CONVERGED ? GBPA_SUCCESS : rc;
   }
   gbpa_operator *Ac = M->ops[level - 1];
   T *Xc = (T *)M->X[level - 1], *Yc = (T *)M->Y[level - 1];
   // pre-smooth from a zero guess: Y = S X
   int rc = chebyshev_mult<T>(M->sm[level], X, Y);
   // residual R = X - A Y, restricted to the coarse right-hand side
   if (!rc) { rc = gbpa_operator_mult(A, Y, R); }
   if (!rc) { rc = axpby<T>(ctx, n, 1.0, X, -1.0, R); }
   if (!rc) { rc = ptransfer_mult_transpose<T>(M->P[level - 1], R, Xc); }
   if (!rc) { rc = fill<T>(ctx, Ac->d.ndofs, 0.0, Yc); }
   if (!rc) { rc = mg_cycle<T>(M, level - 1); }
   // prolongate and add
   if (!rc) { rc = ptransfer_mult<T>(M->P[level - 1], Yc, Z); }
   if (!rc) { rc = axpby<T>(ctx, n, 1.0, Z, 1.0, Y); }
   // post-smooth: Y += S (X - A Y)
   if (!rc) { rc = gbpa_operator_mult(A, Y, R); }
   if (!rc) { rc = axpby<T>(ctx, n, 1.0, X, -1.0, R); }
   if (!rc) { rc = chebyshev_mult<T>(M->sm[level], R, Z); }
   if (!rc) { rc = axpby<T>(ctx, n, 1.0, Z, 1.0, Y); }
   return rc;
}

// y = V-cycle(x) with x, y in the levels' vector type
template <typename T>
int mg_mult(gbpa_multigrid *M, const T *x, T *y)
{
   const int top = M->nl - 1;
   const int64_t n = M->ops[top]->d.ndofs;
   int rc = check_cuda(cudaMemcpyAsync(M->X[top], x, sizeof(T) * n, cudaMemcpyDeviceToDevice, M->ctx->stream), "copy");
   if (!rc) { rc = fill<T>(M->ctx, n, 0.0, (T *)M->Y[top]); }
   if (!rc) { rc = mg_cycle<T>(M, top); }
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(y, M->Y[top], sizeof(T) * n, cudaMemcpyDeviceToDevice, M->ctx->stream), "copy"); }
   return rc;
}

// z = V-cycle(r) for FP64 vectors r, z whatever the levels' type (FP32
// levels: r narrowed into the top level's right-hand side, the correction
// widened back)
int mg_precondition(gbpa_multigrid *M, const double *r, double *z)
{
   if (!M->f32) { return mg_mult<double>(M, r, z); }
   const int top = M->nl - 1;
   const int64_t n = M->ops[top]->d.ndofs;
   gbpa_ctx *ctx = M->ctx;
   mg_convert_kernel<float><<<vgrid(ctx, n), 256, 0, ctx->stream>>>(n, r, (float *)M->X[top]);
   int rc = last_launch(ctx, "mg_convert");
   if (!rc) { rc = fill<float>(ctx, n, 0.0, (float *)M->Y[top]); }
   if (!rc) { rc = mg_cycle<float>(M, top); }
   if (!rc)
   {
      mg_widen_kernel<float><<<vgrid(ctx, n), 256, 0, ctx->stream>>>(n, (const float *)M->Y[top], z);
      rc = last_launch(ctx, "mg_widen");
   }
   return rc;
}
} // namespace

// ------------------------------------------------------------ p-transfer
extern "C" int gbpa_ptransfer_create(gbpa_ctx_t ctx, int ne, int d1d_c, int ndofs_c, const int *gather_map_c,
                                     const int *offsets_c, const int *indices_c, int d1d_f, int ndofs_f,
                                     const int *gather_map_f, const int *offsets_f, const int *indices_f,
                                     const double *Bi, int precision, gbpa_ptransfer_t *out)
{
   if (!ctx || !out || ne < 0 || ndofs_c < 0 || ndofs_f < 0 || d1d_c < 1 || d1d_f < 1) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (precision != GBPA_F64 && precision != GBPA_F32) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (d1d_c > MG_MAX_1D || d1d_f > MG_MAX_1D) { return GBPA_ERR_UNSUPPORTED; }
   if (ne > 0 && (!gather_map_c || !offsets_c || !indices_c || !gather_map_f || !offsets_f || !indices_f || !Bi))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   gbpa_ptransfer *T = new (std::nothrow) gbpa_ptransfer;
   if (!T) { return GBPA_ERR_OUT_OF_MEMORY; }
   T->ctx = ctx; T->ne = ne; T->dc = d1d_c; T->df = d1d_f; T->ndofs_c = ndofs_c; T->ndofs_f = ndofs_f;
   T->f32 = precision == GBPA_F32;
   T->gm_c = gather_map_c; T->off_c = offsets_c; T->ind_c = indices_c; T->gm_f = gather_map_f;
   const int64_t nf = (int64_t)ne * d1d_f * d1d_f * d1d_f, nc = (int64_t)ne * d1d_c * d1d_c * d1d_c;
   const int nb = d1d_f * d1d_c;
   std::vector<float> b32(Bi ? nb : 0);
   for (int i = 0; Bi && i < nb; ++i) { b32[i] = (float)Bi[i]; }
   const void *src = T->f32 ? (const void *)b32.data() : (const void *)Bi;
   int rc = dev_alloc(&T->Bi, vbytes(T->f32) * nb);
   if (!rc && Bi) { rc = check_cuda(cudaMemcpy(T->Bi, src, vbytes(T->f32) * nb, cudaMemcpyHostToDevice), "copy"); }
   if (!rc) { rc = dev_alloc((void **)&T->own, nf); }
   if (!rc) { rc = check_cuda(cudaMemsetAsync(T->own, 0, nf > 0 ? nf : 1, ctx->stream), "memset"); }
   if (!rc) { rc = dev_alloc(&T->yEc, vbytes(T->f32) * nc); }
   if (!rc && ndofs_f > 0)
   {
      mg_owner_kernel<<<grid_for(ndofs_f, 256), 256, 0, ctx->stream>>>(ndofs_f, offsets_f, indices_f, T->own);
      rc = last_launch(ctx, "mg_owner");
   }
   if (rc) { gbpa_ptransfer_destroy(T); return rc; }
   *out = T;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_ptransfer_destroy(gbpa_ptransfer_t T)
{
   if (!T) { return GBPA_SUCCESS; }
   cudaStreamSynchronize(T->ctx->stream);
   cudaFree(T->Bi); cudaFree(T->own); cudaFree(T->yEc);
   delete T;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_ptransfer_mult(gbpa_ptransfer_t T, const void *xc, void *yf)
{
   if (!T || (T->ne > 0 && (!xc || !yf))) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (T->ne == 0) { return GBPA_SUCCESS; }
   return T->f32 ? ptransfer_mult<float>(T, (const float *)xc, (float *)yf)
                 : ptransfer_mult<double>(T, (const double *)xc, (double *)yf);
}

extern "C" int gbpa_ptransfer_mult_transpose(gbpa_ptransfer_t T, const void *xf, void *yc)
{
   if (!T || (T->ne > 0 && (!xf || !yc))) { return GBPA_ERR_INVALID_ARGUMENT; }
   return T->f32 ? ptransfer_mult_transpose<float>(T, (const float *)xf, (float *)yc)
                 : ptransfer_mult_transpose<double>(T, (const double *)xf, (double *)yc);
}

// --------------------------------------------------------------- Chebyshev
extern "C" int gbpa_chebyshev_create(gbpa_operator_t A, const double *diag, int order, double max_eig,
                                     int power_iterations, double power_tol, unsigned long long seed,
                                     gbpa_chebyshev_t *out)
{
   if (!A || !out || (A->d.ndofs > 0 && !diag) || order < 1 || order > 8 || power_iterations < 0)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   gbpa_ctx *ctx = A->ctx;
   const int n = A->d.ndofs;
   gbpa_chebyshev *S = new (std::nothrow) gbpa_chebyshev;
   if (!S) { return GBPA_ERR_OUT_OF_MEMORY; }
   S->A = A; S->order = order; S->f32 = fp32_vectors(A);
   const size_t vb = vbytes(S->f32) * (size_t)n;
   int rc = dev_alloc(&S->dinv, vb);
   if (!rc) { rc = dev_alloc(&S->res, vb); }
   if (!rc) { rc = dev_alloc(&S->h, vb); }
   // dinv = 1/diag, 1 on the essential dofs (linalg/solvers.cpp:540-550)
   if (!rc && n > 0)
   {
      if (S->f32) { mg_dinv_kernel<float><<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(n, diag, (float *)S->dinv); }
      else { mg_dinv_kernel<double><<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(n, diag, (double *)S->dinv); }
      rc = last_launch(ctx, "mg_dinv");
   }
   if (!rc && A->d.n_ess > 0)
   {
      if (S->f32) { mg_set_ess_kernel<float><<<grid_for(A->d.n_ess, 256), 256, 0, ctx->stream>>>(A->d.n_ess, A->d.ess, 1.0f, (float *)S->dinv); }
      else { mg_set_ess_kernel<double><<<grid_for(A->d.n_ess, 256), 256, 0, ctx->stream>>>(A->d.n_ess, A->d.ess, 1.0, (double *)S->dinv); }
      rc = last_launch(ctx, "mg_set_ess");
   }
   if (!rc && max_eig <= 0.0)
   {
      rc = S->f32 ? power_method<float>(S, power_iterations, power_tol, seed, &max_eig)
                  : power_method<double>(S, power_iterations, power_tol, seed, &max_eig);
   }
   if (rc) { gbpa_chebyshev_destroy(S); return rc; }
   if (!(max_eig > 0.0) || !std::isfinite(max_eig)) { gbpa_chebyshev_destroy(S); return GBPA_ERR_NOT_FINITE; }
   S->lambda = max_eig;
   chebyshev_coeffs(order, max_eig, S->coeffs);
   *out = S;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_chebyshev_destroy(gbpa_chebyshev_t S)
{
   if (!S) { return GBPA_SUCCESS; }
   cudaStreamSynchronize(S->A->ctx->stream);
   cudaFree(S->dinv); cudaFree(S->res); cudaFree(S->h);
   delete S;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_chebyshev_get_max_eig(gbpa_chebyshev_t S, double *max_eig)
{
   if (!S || !max_eig) { return GBPA_ERR_INVALID_ARGUMENT; }
   *max_eig = S->lambda;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_chebyshev_mult(gbpa_chebyshev_t S, const void *x, void *y)
{
   if (!S || (S->A->d.ndofs > 0 && (!x || !y))) { return GBPA_ERR_INVALID_ARGUMENT; }
   return S->f32 ? chebyshev_mult<float>(S, (const float *)x, (float *)y)
                 : chebyshev_mult<double>(S, (const double *)x, (double *)y);
}

// -------------------------------------------------------------- multigrid
extern "C" int gbpa_multigrid_create(gbpa_ctx_t ctx, int nlevels, const gbpa_operator_t *ops,
                                     const gbpa_chebyshev_t *smoothers, const gbpa_ptransfer_t *prolongations,
                                     double coarse_rel_tol, int coarse_max_it, int coarse_jacobi,
                                     const double *coarse_diag, gbpa_multigrid_t *out)
{
   if (!ctx || !out || nlevels < 1 || !ops || (nlevels > 1 && (!smoothers || !prolongations)) ||
       coarse_rel_tol < 0 || coarse_max_it < 0 || (coarse_jacobi != 0 && coarse_jacobi != 1) || !ops[0])
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   const bool f32 = fp32_vectors(ops[0]);
   for (int l = 0; l < nlevels; ++l)
   {
      if (!ops[l] || ops[l]->ctx != ctx || fp32_vectors(ops[l]) != f32) { return GBPA_ERR_INVALID_ARGUMENT; }
      if (ops[l]->d.kind != GBPA_DIFFUSION) { return GBPA_ERR_UNSUPPORTED; }
      if (l > 0)
      {
         const gbpa_ptransfer *P = prolongations[l - 1];
         if (!smoothers[l] || smoothers[l]->A != ops[l] || !P || P->f32 != f32) { return GBPA_ERR_INVALID_ARGUMENT; }
         if (P->ndofs_c != ops[l - 1]->d.ndofs || P->ndofs_f != ops[l]->d.ndofs) { return GBPA_ERR_INVALID_ARGUMENT; }
      }
   }
   // the Jacobi coarse CG needs the coarse diagonal: given, or assembled by
   // an operator with FP64 data
   if (coarse_jacobi && !coarse_diag && f32) { return GBPA_ERR_INVALID_ARGUMENT; }
   gbpa_multigrid *M = new (std::nothrow) gbpa_multigrid;
   if (!M) { return GBPA_ERR_OUT_OF_MEMORY; }
   M->ctx = ctx; M->nl = nlevels; M->f32 = f32;
   M->coarse_tol = coarse_rel_tol; M->coarse_max = coarse_max_it;
   int rc = GBPA_SUCCESS;
   for (int l = 0; l < nlevels && !rc; ++l)
   {
      const size_t vb = vbytes(f32) * (size_t)ops[l]->d.ndofs;
      M->ops.push_back(ops[l]);
      M->sm.push_back(l > 0 ? smoothers[l] : nullptr);
      if (l > 0) { M->P.push_back(prolongations[l - 1]); }
      void *x = nullptr, *y = nullptr, *r = nullptr, *z = nullptr;
      rc = dev_alloc(&x, vb);
      if (!rc) { rc = dev_alloc(&y, vb); }
      if (!rc) { rc = dev_alloc(&r, vb); }
      if (!rc) { rc = dev_alloc(&z, vb); }
      M->X.push_back(x); M->Y.push_back(y); M->R.push_back(r); M->Z.push_back(z);
   }
   const int64_t n0 = ops[0]->d.ndofs;
   if (!rc) { rc = dev_alloc(&M->coarse_dinv, vbytes(f32) * n0); }
   if (!rc && !coarse_jacobi)
   {
      rc = f32 ? fill<float>(ctx, n0, 1.0, (float *)M->coarse_dinv) : fill<double>(ctx, n0, 1.0, (double *)M->coarse_dinv);
   }
   if (!rc && coarse_jacobi && n0 > 0)
   {
      // OperatorJacobiSmoother on the coarse constrained operator: its
      // diagonal (1 on the essential dofs), inverted
      double *diag = nullptr, *dinv64 = nullptr;
      rc = dev_alloc((void **)&dinv64, sizeof(double) * n0);
      if (!rc && !coarse_diag)
      {
         rc = dev_alloc((void **)&diag, sizeof(double) * n0);
         if (!rc) { rc = gbpa_operator_assemble_diagonal(ops[0], diag); }
      }
      if (!rc)
      {
         rc = gbpa_jacobi_setup(ctx, n0, coarse_diag ? coarse_diag : diag, ops[0]->d.ess, ops[0]->d.n_ess, 1.0,
                                dinv64);
      }
      if (!rc)
      {
         if (f32)
         {
            mg_convert_kernel<float><<<vgrid(ctx, n0), 256, 0, ctx->stream>>>(n0, dinv64, (float *)M->coarse_dinv);
            rc = last_launch(ctx, "mg_convert");
         }
         else
         {
            rc = check_cuda(cudaMemcpyAsync(M->coarse_dinv, dinv64, sizeof(double) * n0, cudaMemcpyDeviceToDevice,
                                            ctx->stream), "copy");
         }
      }
      if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
      cudaFree(diag); cudaFree(dinv64);
   }
   if (!rc) { rc = dev_alloc((void **)&M->d_dot, sizeof(double)); }
   if (rc) { gbpa_multigrid_destroy(M); return rc; }
   *out = M;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_multigrid_destroy(gbpa_multigrid_t M)
{
   if (!M) { return GBPA_SUCCESS; }
   cudaStreamSynchronize(M->ctx->stream);
   for (void *p : M->X) { cudaFree(p); }
   for (void *p : M->Y) { cudaFree(p); }
   for (void *p : M->R) { cudaFree(p); }
   for (void *p : M->Z) { cudaFree(p); }
   cudaFree(M->coarse_dinv); cudaFree(M->d_dot);
   delete M;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_multigrid_mult(gbpa_multigrid_t M, const void *x, void *y)
{
   if (!M || (M->ops[M->nl - 1]->d.ndofs > 0 && (!x || !y))) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (M->ops[M->nl - 1]->d.ndofs == 0) { return GBPA_SUCCESS; }
   return M->f32 ? mg_mult<float>(M, (const float *)x, (float *)y)
                 : mg_mult<double>(M, (const double *)x, (double *)y);
}

// CGSolver::Mult (linalg/solvers.cpp:869-1050) preconditioned by the V-cycle,
// zero initial guess; the stopping rule (B r, r) <= max(rel^2 (B r0, r0), abs^2).
// A has FP64 vectors; the multigrid levels may run in FP32 (the V-cycle is
// then an FP32 preconditioner of the FP64 iteration).
extern "C" int gbpa_pcg_solve_mg(gbpa_operator_t A, gbpa_multigrid_t M, const double *b, double *x, double rel_tol,
                                 double abs_tol, int max_it, gbpa_solve_info *info)
{
   if (!A || !M || fp32_vectors(A) || A->ctx != M->ctx || M->ops[M->nl - 1]->d.ndofs != A->d.ndofs ||
       (A->d.ndofs > 0 && (!b || !x)) || max_it < 0 || rel_tol < 0 || abs_tol < 0)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   gbpa_ctx *ctx = A->ctx;
   const int64_t n = A->d.ndofs;
   double *r = nullptr, *d = nullptr, *z = nullptr;
   int rc = dev_alloc((void **)&r, sizeof(double) * n);
   if (!rc) { rc = dev_alloc((void **)&d, sizeof(double) * n); }
   if (!rc) { rc = dev_alloc((void **)&z, sizeof(double) * n); }
   StreamTimer timer(ctx->stream);
   M->coarse_iterations = 0;
   int final_iter = 0, converged = 0, status = GBPA_SUCCESS;
   double nom = 0.0, nom0 = 0.0, den = 0.0, betanom = 0.0;
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream), "copy"); }
   if (!rc) { rc = fill<double>(ctx, n, 0.0, x); }
   if (!rc) { rc = mg_precondition(M, r, z); }
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(d, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream), "copy"); }
   if (!rc) { rc = host_dot<double>(ctx, n, d, r, M->d_dot, &nom); }
   nom0 = nom;
   if (!rc)
   {
      const double r0 = std::fmax(nom * rel_tol * rel_tol, abs_tol * abs_tol);
      betanom = nom;
      if (!std::isfinite(nom)) { status = GBPA_ERR_NOT_FINITE; }
      else if (nom < 0.0) { status = GBPA_SUCCESS; }
      else if (nom <= r0) { converged = 1; }
      else
      {
         rc = gbpa_operator_mult(A, d, z);
         if (!rc) { rc = host_dot<double>(ctx, n, z, d, M->d_dot, &den); }
         final_iter = den == 0.0 ? 0 : max_it;
         for (int i = 1; !rc && den != 0.0;)
         {
            const double alpha = nom / den;
            rc = axpby<double>(ctx, n, alpha, d, 1.0, x);
            if (!rc) { rc = axpby<double>(ctx, n, -alpha, z, 1.0, r); }
            if (!rc) { rc = mg_precondition(M, r, z); }
            if (!rc) { rc = host_dot<double>(ctx, n, r, z, M->d_dot, &betanom); }
            if (rc) { break; }
            if (!std::isfinite(betanom)) { status = GBPA_ERR_NOT_FINITE; final_iter = i; break; }
            if (betanom < 0.0) { final_iter = i; break; }
            if (betanom <= r0) { converged = 1; final_iter = i; break; }
            if (++i > max_it) { break; }
            const double beta = betanom / nom;
            rc = axpby<double>(ctx, n, 1.0, z, beta, d);
            if (!rc) { rc = gbpa_operator_mult(A, d, z); }
            if (!rc) { rc = host_dot<double>(ctx, n, d, z, M->d_dot, &den); }
            if (!rc && den == 0.0) { final_iter = i; }
            nom = betanom;
         }
      }
   }
   const float ms = timer.stop(ctx->stream);
   cudaFree(r); cudaFree(d); cudaFree(z);
   if (info)
   {
      info->iterations = final_iter;
      info->converged = converged;
      info->initial_norm = nom0 >= 0 ? std::sqrt(nom0) : nom0;
      info->final_norm = betanom >= 0 ? std::sqrt(betanom) : betanom;
      info->true_rel_residual = -1.0;
      info->outer_iterations = final_iter;
      info->inner_iterations = (int)M->coarse_iterations;
      info->seconds = ms * 1e-3;
   }
   if (rc) { return rc; }
   if (status) { return status; }
   return converged ? GBPA_SUCCESS : GBPA_ERR_NOT_CONVERGED;
}
