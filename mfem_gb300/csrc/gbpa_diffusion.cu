// Diffusion PA kernels: apply (E->E and gather-fused), diagonal, and their
// C-ABI entry points. Reference: fem/integ/bilininteg_diffusion_pa.cpp,
// fem/integ/bilininteg_diffusion_kernels.hpp.
#include "gbpa_dispatch.cuh"

namespace gbpa
{

// Diagonal (2D slab). For pair (i, j) of gradient directions the element
// diagonal gains sum_q L_i O_ij R_j where, per direction t, the 1D factor is
// B^2, B*G or G^2 depending on whether t equals i and/or j
// (fem/integ/bilininteg_diffusion_kernels.hpp:268-485). With symmetric qdata
// the (i, j) and (j, i) terms are equal, so off-diagonal pairs are done once
// with weight 2.
template <int TD, int TQ>
__global__ void diffusion_diagonal_kernel(int ne, int symm, int d1d, int q1d,
                                          const double *__restrict__ gB,
                                          const double *__restrict__ gG,
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
   double *tab = reinterpret_cast<double *>(smem_raw);   // BB | BG | GG, each [Q][D]
   double *QQD = tab + 3 * Q * D + tz * (2 * D * Q * Q);  // [dz][qy][qx]
   double *QDD = QQD + D * Q * Q;                          // [dz][dy][qx]
   const int tid = tx + Q * (ty + Q * tz), nthr = Q * Q * blockDim.z;
   for (int i = tid; i < Q * D; i += nthr)
   {
      const int q = i % Q, d = i / Q;
      const double b = gB[i], g = gG[i];
      tab[q * D + d] = b * b;
      tab[Q * D + q * D + d] = b * g;
      tab[2 * Q * D + q * D + d] = g * g;
   }
   __syncthreads();
   const int S = symm ? 6 : 9;
   const double *qe = qd + (long long)e * S * Q3 + tx + Q * ty;
   double acc[DM];
#pragma unroll
   for (int dz = 0; dz < DM; ++dz) { acc[dz] = 0.0; }
   for (int i = 0; i < 3; ++i)
   {
      for (int j = symm ? i : 0; j < 3; ++j)
      {
         int k;
         if (symm) { k = j >= i ? 3 - (3 - i) * (2 - i) / 2 + j : 3 - (3 - j) * (2 - j) / 2 + i; }
         else { k = 3 * i + j; }
         const double w = (symm && i != j) ? 2.0 : 1.0;
         const double *tz_tab = tab + Q * D * ((i == 2) + (j == 2));
         const double *ty_tab = tab + Q * D * ((i == 1) + (j == 1));
         const double *tx_tab = tab + Q * D * ((i == 0) + (j == 0));
         // z (registers): QQD[dz][qy][qx] = sum_qz tab_z[qz][dz] O(qx,qy,qz)
         double s[DM];
#pragma unroll
         for (int dz = 0; dz < DM; ++dz) { s[dz] = 0.0; }
#pragma unroll
         for (int qz = 0; qz < QM; ++qz)
         {
            if (qz >= Q) { break; }
            const double O = active ? __ldg(qe + Q * Q * qz + (long long)k * Q3) : 0.0;
#pragma unroll
            for (int dz = 0; dz < DM; ++dz)
            {
               if (dz >= D) { break; }
               s[dz] += tz_tab[qz * D + dz] * O;
            }
         }
#pragma unroll
         for (int dz = 0; dz < DM; ++dz)
         {
            if (dz >= D) { break; }
            QQD[(dz * Q + ty) * Q + tx] = s[dz];
         }
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
                  t += ty_tab[qy * D + dy] * QQD[(dz * Q + qy) * Q + tx];
               }
               QDD[(dz * D + dy) * Q + tx] = t;
            }
         }
         __syncthreads();
         if (tx < D && ty < D)
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
                  t += tx_tab[qx * D + tx] * QDD[(dz * D + ty) * Q + qx];
               }
               acc[dz] += w * t;
            }
         }
      }
   }
   if (active && tx < D && ty < D)
   {
      const long long base = (long long)e * D * D * D;
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         y[base + tx + D * (ty + D * dz)] += acc[dz];
      }
   }
}

static const void *diagonal_kernel(int D, int Q)
{
#define GBPA_CASE(d, q) \
   if (D == d && Q == q) { return (const void *)diffusion_diagonal_kernel<d, q>; }
   GBPA_DQ_LIST(GBPA_CASE)
#undef GBPA_CASE
   return (const void *)diffusion_diagonal_kernel<0, 0>;
}

int launch_diffusion_diagonal(gbpa_ctx *ctx, int ne, int symm, int D, int Q,
                              const double *B, const double *G,
                              const double *qd, double *y)
{
   if (ne == 0) { return GBPA_SUCCESS; }
   if (D > Q)
   {
      // the x-stage maps thread (tx, ty) to (dx, dy); it needs D <= Q
      return GBPA_ERR_UNSUPPORTED;
   }
   int nbz = 256 / (Q * Q);
   if (nbz < 1) { nbz = 1; }
   const size_t smem = sizeof(double) * (3 * Q * D + (size_t)nbz * 2 * D * Q * Q);
   const void *k = diagonal_kernel(D, Q);
   void *args[] = {&ne, &symm, &D, &Q, (void *)&B, (void *)&G, (void *)&qd, &y};
   return launch_generic(ctx, k, dim3((ne + nbz - 1) / nbz), dim3(Q, Q, nbz),
                         args, smem, "diffusion_diagonal");
}

} // namespace gbpa

using namespace gbpa;

static bool dq_ok(int D, int Q)
{
   return D >= 1 && Q >= 1 && D <= GBPA_MAX_1D && Q <= GBPA_MAX_1D;
}

extern "C" int gbpa_diffusion_apply3d(gbpa_ctx_t ctx, int ne, int symm,
                                      int d1d, int q1d, const double *B,
                                      const double *G, const double *Bt,
                                      const double *Gt, const double *D,
                                      const double *x, double *y)
{
   (void)Bt; (void)Gt;
   if (!ctx || ne < 0 || (ne > 0 && (!B || !G || !D || !x || !y)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (!dq_ok(d1d, q1d)) { return GBPA_ERR_UNSUPPORTED; }
   return launch_diffusion_apply<double>(ctx, ne, symm ? 1 : 0, d1d, q1d, B, G,
                                         D, x, nullptr, nullptr, y, true);
}

extern "C" int gbpa_diffusion_apply3d_f32(gbpa_ctx_t ctx, int ne, int symm,
                                          int d1d, int q1d, const float *B,
                                          const float *G, const float *D,
                                          const float *x, float *y)
{
   if (!ctx || ne < 0 || (ne > 0 && (!B || !G || !D || !x || !y)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (!dq_ok(d1d, q1d)) { return GBPA_ERR_UNSUPPORTED; }
   return launch_diffusion_apply<float>(ctx, ne, symm ? 1 : 0, d1d, q1d, B, G,
                                        D, x, nullptr, nullptr, y, true);
}

extern "C" int gbpa_diffusion_diagonal3d(gbpa_ctx_t ctx, int ne, int symm,
                                         int d1d, int q1d, const double *B,
                                         const double *G, const double *D,
                                         double *y)
{
   if (!ctx || ne < 0 || (ne > 0 && (!B || !G || !D || !y)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (!dq_ok(d1d, q1d)) { return GBPA_ERR_UNSUPPORTED; }
   return launch_diffusion_diagonal(ctx, ne, symm ? 1 : 0, d1d, q1d, B, G, D, y);
}

// VectorDiffusionIntegrator::AddMultPA, 3D, scalar or vector coefficient
// (fem/integ/bilininteg_vecdiffusion_pa.cpp:282-330, kernel
// fem/integ/bilininteg_vecdiffusion_pa.hpp:96-163): the scalar symmetric
// apply on the vdim NE pseudo-elements of the (D^3, vdim, NE) E-vectors
extern "C" int gbpa_vector_diffusion_apply3d(gbpa_ctx_t ctx, int ne, int vdim, int d1d, int q1d,
                                             const double *B, const double *G, const double *D,
                                             const double *x, double *y)
{
   if (!ctx || ne < 0 || vdim < 1 || vdim > 3) { return GBPA_ERR_INVALID_ARGUMENT; }
   return gbpa_diffusion_apply3d(ctx, ne * vdim, 1, d1d, q1d, B, G, nullptr, nullptr, D, x, y);
}
