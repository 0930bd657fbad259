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
