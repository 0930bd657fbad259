// Mass PA kernels: apply (E->E and gather-fused), diagonal, setup entry
// points. Reference: fem/integ/bilininteg_mass_pa.cpp,
// fem/integ/bilininteg_mass_kernels.hpp.
#include "gbpa_dispatch.cuh"

namespace gbpa
{

// Diagonal: sum_q B^2 (x) B^2 (x) B^2 . D, contracted z, y, x
// (fem/integ/bilininteg_mass_kernels.hpp:262-416).
template <int TD, int TQ>
__global__ void mass_diagonal_kernel(int ne, int d1d, int q1d,
                                     const double *__restrict__ gB,
                                     const double *__restrict__ qd,
                                     double *__restrict__ y)
{
   constexpr int DM = TD ? TD : GBPA_MAX_1D;
   constexpr int QM = TQ ? TQ : GBPA_MAX_1D;
   const int D = TD ? TD : d1d, Q = TQ ? TQ : q1d;
   const int Q3 = Q * Q * Q;
   const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
   const int e = blockIdx.x * blockDim.z + tz;
   const bool active = e < ne;
   extern __shared__ __align__(16) unsigned char smem_raw[];
   double *BB = reinterpret_cast<double *>(smem_raw);
   double *QQD = BB + Q * D + tz * (2 * D * Q * Q);
   double *QDD = QQD + D * Q * Q;
   const int tid = tx + Q * (ty + Q * tz), nthr = Q * Q * blockDim.z;
   for (int i = tid; i < Q * D; i += nthr)
   {
      const double b = gB[i];
      BB[(i % Q) * D + i / Q] = b * b;
   }
   __syncthreads();
   const double *qe = qd + (long long)e * Q3 + tx + Q * ty;
   double s[DM];
#pragma unroll
   for (int dz = 0; dz < DM; ++dz) { s[dz] = 0.0; }
#pragma unroll
   for (int qz = 0; qz < QM; ++qz)
   {
      if (qz >= Q) { break; }
      const double O = active ? __ldg(qe + Q * Q * qz) : 0.0;
#pragma unroll
      for (int dz = 0; dz < DM; ++dz) { if (dz >= D) { break; } s[dz] += BB[qz * D + dz] * O; }
   }
#pragma unroll
   for (int dz = 0; dz < DM; ++dz) { if (dz >= D) { break; } QQD[(dz * Q + ty) * Q + tx] = s[dz]; }
   __syncthreads();
   for (int dy = ty; dy < D; dy += Q)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         double t = 0.0;
#pragma unroll
         for (int qy = 0; qy < QM; ++qy)
         {
            if (qy >= Q) { break; }
            t += BB[qy * D + dy] * QQD[(dz * Q + qy) * Q + tx];
         }
         QDD[(dz * D + dy) * Q + tx] = t;
      }
   }
   __syncthreads();
   if (active)
   {
      const long long base = (long long)e * D * D * D;
      for (int dy = ty; dy < D; dy += Q)
         for (int dx = tx; dx < D; dx += Q)
         {
#pragma unroll
            for (int dz = 0; dz < DM; ++dz)
            {
               if (dz >= D) { break; }
               double t = 0.0;
#pragma unroll
               for (int qx = 0; qx < QM; ++qx)
               {
                  if (qx >= Q) { break; }
                  t += BB[qx * D + dx] * QDD[(dz * D + dy) * Q + qx];
               }
               y[base + dx + D * (dy + D * dz)] += t;
            }
         }
   }
}

static const void *mass_diag_kernel(int D, int Q)
{
#define GBPA_CASE(d, q) \
   if (D == d && Q == q) { return (const void *)mass_diagonal_kernel<d, q>; }
   GBPA_DQ_LIST(GBPA_CASE)
#undef GBPA_CASE
   return (const void *)mass_diagonal_kernel<0, 0>;
}

int launch_mass_diagonal(gbpa_ctx *ctx, int ne, int D, int Q, const double *B,
                         const double *qd, double *y)
{
   if (ne == 0) { return GBPA_SUCCESS; }
   int nbz = 256 / (Q * Q);
   if (nbz < 1) { nbz = 1; }
   const size_t smem = sizeof(double) * (Q * D + (size_t)nbz * 2 * D * Q * Q);
   void *args[] = {&ne, &D, &Q, (void *)&B, (void *)&qd, &y};
   return launch_generic(ctx, mass_diag_kernel(D, Q), dim3((ne + nbz - 1) / nbz),
                         dim3(Q, Q, nbz), args, smem, "mass_diagonal");
}

} // namespace gbpa

using namespace gbpa;

static bool dq_ok(int D, int Q)
{
   return D >= 1 && Q >= 1 && D <= GBPA_MAX_1D && Q <= GBPA_MAX_1D;
}

extern "C" int gbpa_mass_apply3d(gbpa_ctx_t ctx, int ne, int d1d, int q1d,
                                 const double *B, const double *Bt,
                                 const double *D, const double *x, double *y)
{
   (void)Bt;
   if (!ctx || ne < 0 || (ne > 0 && (!B || !D || !x || !y)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (!dq_ok(d1d, q1d)) { return GBPA_ERR_UNSUPPORTED; }
   return launch_mass_apply<double>(ctx, ne, d1d, q1d, B, D, x, nullptr, nullptr, y, true);
}

extern "C" int gbpa_mass_apply3d_f32(gbpa_ctx_t ctx, int ne, int d1d, int q1d,
                                     const float *B, const float *D,
                                     const float *x, float *y)
{
   if (!ctx || ne < 0 || (ne > 0 && (!B || !D || !x || !y)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (!dq_ok(d1d, q1d)) { return GBPA_ERR_UNSUPPORTED; }
   return launch_mass_apply<float>(ctx, ne, d1d, q1d, B, D, x, nullptr, nullptr, y, true);
}

extern "C" int gbpa_mass_diagonal3d(gbpa_ctx_t ctx, int ne, int d1d, int q1d,
                                    const double *B, const double *D, double *y)
{
   if (!ctx || ne < 0 || (ne > 0 && (!B || !D || !y)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (!dq_ok(d1d, q1d)) { return GBPA_ERR_UNSUPPORTED; }
   return launch_mass_diagonal(ctx, ne, d1d, q1d, B, D, y);
}

// ------------------------------------------------------------ linear form
namespace gbpa
{
// DLFEvalAssemble3D (fem/integ/lininteg_domain_kernels.hpp:164-...): one
// element per block of M x M threads (M = max(D, Q)); the quadrature values
// v = W f detJ in shared memory, then the transposed contractions x, y, z.
__global__ void domain_lf_kernel(int ne, int D, int Q, const double *__restrict__ B, const double *__restrict__ W,
                                 const double *__restrict__ detJ, const double *__restrict__ f, int64_t c_size,
                                 double *__restrict__ yE)
{
   extern __shared__ double sm[];
   const int e = blockIdx.x;
   const int tx = threadIdx.x, ty = threadIdx.y, M = blockDim.x;
   const int Q3 = Q * Q * Q, D3 = D * D * D;
   double *sB = sm;                  // [Q][D] as B(q, d) = B[q + Q d]
   double *v = sB + Q * D;           // [Q^3]
   double *t1 = v + Q3;              // [Q][Q][D]
   double *t2 = t1 + Q * Q * D;      // [Q][D][D]
   for (int i = tx + M * ty; i < Q * D; i += M * M) { sB[i] = B[i]; }
   if (tx < Q && ty < Q)
   {
      for (int qz = 0; qz < Q; ++qz)
      {
         const int q = tx + Q * (ty + Q * qz);
         const long long k = (long long)e * Q3 + q;
         v[q] = W[q] * (c_size == 1 ? f[0] : f[k]) * detJ[k];
      }
   }
   __syncthreads();
   if (tx < D && ty < Q)   // x: thread (dx, qy)
   {
      for (int qz = 0; qz < Q; ++qz)
      {
         double s = 0.0;
         for (int qx = 0; qx < Q; ++qx) { s += sB[qx + Q * tx] * v[qx + Q * (ty + Q * qz)]; }
         t1[tx + D * (ty + Q * qz)] = s;
      }
   }
   __syncthreads();
   if (tx < D && ty < D)   // y: thread (dx, dy)
   {
      for (int qz = 0; qz < Q; ++qz)
      {
         double s = 0.0;
         for (int qy = 0; qy < Q; ++qy) { s += sB[qy + Q * ty] * t1[tx + D * (qy + Q * qz)]; }
         t2[tx + D * (ty + D * qz)] = s;
      }
   }
   __syncthreads();
   if (tx < D && ty < D)   // z
   {
      for (int dz = 0; dz < D; ++dz)
      {
         double s = 0.0;
         for (int qz = 0; qz < Q; ++qz) { s += sB[qz + Q * dz] * t2[tx + D * (ty + D * qz)]; }
         yE[(long long)e * D3 + tx + D * (ty + D * dz)] = s;
      }
   }
}
} // namespace gbpa

// DomainLFIntegrator::AssembleDevice + LinearFormExtension::Assemble
// (fem/integ/lininteg_domain.cpp:22-59, fem/linearform_ext.cpp:20-68)
extern "C" int gbpa_domain_lf3d(gbpa_ctx_t ctx, int ne, int d1d, int q1d, const double *B, const double *W,
                                const double *detJ, const double *coeff, int64_t coeff_size, int ndofs,
                                const int *offsets, const int *indices, double *b)
{
   if (!ctx || ne < 0 || ndofs < 0 || (ne > 0 && (!B || !W || !detJ || !coeff || !offsets || !indices)) ||
       (ndofs > 0 && !b))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (!dq_ok(d1d, q1d)) { return GBPA_ERR_UNSUPPORTED; }
   if (coeff_size != 1 && coeff_size != (int64_t)ne * q1d * q1d * q1d) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (ndofs == 0) { return GBPA_SUCCESS; }
   const int64_t nE = (int64_t)ne * d1d * d1d * d1d;
   double *yE = (double *)scratch(ctx, SLOT_EVEC_A, sizeof(double) * (nE > 0 ? nE : 1));
   if (!yE) { return GBPA_ERR_OUT_OF_MEMORY; }
   if (ne > 0)
   {
      int D = d1d, Q = q1d, M = d1d > q1d ? d1d : q1d;
      const size_t smem = sizeof(double) * ((size_t)Q * D + (size_t)Q * Q * Q + (size_t)Q * Q * D + (size_t)Q * D * D);
      void *args[] = {&ne, &D, &Q, (void *)&B, (void *)&W, (void *)&detJ, (void *)&coeff, &coeff_size, &yE};
      const int rc = launch_generic(ctx, (const void *)domain_lf_kernel, dim3(ne), dim3(M, M), args, smem,
                                    "domain_lf");
      if (rc) { return rc; }
   }
   return launch_csr_scatter<double>(ctx, ndofs, offsets, indices, yE, b, nullptr, nullptr, false, false);
}

// VectorMassIntegrator::AddMultPA, 3D, scalar or vector coefficient
// (fem/integ/bilininteg_vecmass_pa.cpp:166-210, kernel
// fem/integ/bilininteg_vecmass_pa.hpp:100-...): the scalar mass apply on the
// vdim NE pseudo-elements of the (D^3, vdim, NE) E-vectors; pseudo-element
// c + vdim e reads qdata (c, e) (vector coefficient) or e (scalar one)
extern "C" int gbpa_vector_mass_apply3d(gbpa_ctx_t ctx, int ne, int vdim, int coeff_vdim, int d1d, int q1d,
                                        const double *B, const double *D, const double *x, double *y)
{
   const bool matrix = vdim == 3 && coeff_vdim == 9;
   if (!ctx || ne < 0 || vdim < 1 || vdim > 3 || (coeff_vdim != 1 && coeff_vdim != vdim && !matrix) ||
       (ne > 0 && (!B || !D || !x || !y)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (!dq_ok(d1d, q1d)) { return GBPA_ERR_UNSUPPORTED; }
   if (matrix) { return vector_mass_apply_matrix(ctx, ne, d1d, q1d, B, D, x, y); }
   return launch_mass_apply_qdiv(ctx, ne * vdim, d1d, q1d, B, D, x, y, coeff_vdim == 1 ? vdim : 1);
}
