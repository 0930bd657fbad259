// Sum-factorised 3D diffusion and mass kernels (templated on precision and on
// compile-time (D, Q); TD = TQ = 0 selects the generic runtime-size variant).
//
// Thread layout ("2D slab"): block = (Q, Q, nbz); thread (tx, ty, tz) owns the
// quadrature column (qx = tx, qy = ty) of element blockIdx.x*nbz + tz and keeps
// the z-direction of every intermediate in registers. Only the x- and y-
// contractions exchange data through shared memory, so an element costs four
// block barriers. The contraction sequence is the reference's (x, y, z
// forward; pointwise 3x3 qdata; z, y, x backward; fem/integ/
// bilininteg_diffusion_kernels.hpp:989-1215), reorganised so the z-forward,
// pointwise and z-backward stages fuse into one register loop over qz.
#pragma once
#include "gbpa_internal.cuh"

namespace gbpa
{

template <typename T>
__device__ __forceinline__ T gather_value(const T *__restrict__ x,
                                          const int *__restrict__ gmap,
                                          const unsigned char *__restrict__ mask,
                                          long long slot)
{
   const int g = __ldg(gmap + slot);
   const int j = g >= 0 ? g : -1 - g;
   if (mask && __ldg(mask + j)) { return T(0); }
   const T v = __ldg(x + j);
   return g >= 0 ? v : -v;
}

// Shared memory (in T units) per element for the diffusion apply.
__host__ __device__ inline int diff_smem_per_elem(int D, int Q)
{
   const int a = D * D * D > 3 * D * Q * Q ? D * D * D : 3 * D * Q * Q;
   return a + 2 * D * D * Q;
}
__host__ __device__ inline int mass_smem_per_elem(int D, int Q)
{
   const int a = D * D * D > D * Q * Q ? D * D * D : D * Q * Q;
   return a + D * D * Q;
}

// One element of the diffusion apply for thread (tx, ty) of its Q x Q slab.
// sB/sG: the block's [Q][D] tables in shared memory (already loaded);
// bufA/bufB: this element's shared buffers (diff_smem_per_elem entries).
// part == false: the thread has no slot in the layout and only joins the
// barriers; active == false: the slot's element is past the end (computes
// on zeros, stores nothing). Every thread of the block must call this.
template <typename T, int TD, int TQ, bool GATHER, int MAXD = GBPA_MAX_1D, int MAXQ = GBPA_MAX_1D>
__device__ __forceinline__ void
diffusion_element(long long e, bool active, bool part, int D, int Q, int tx, int ty,
                  int symm, const T *__restrict__ sB, const T *__restrict__ sG,
                  T *__restrict__ bufA, T *__restrict__ bufB, const T *__restrict__ qd,
                  const T *__restrict__ x, const int *__restrict__ gmap,
                  const unsigned char *__restrict__ mask, T *__restrict__ y, int accumulate)
{
   constexpr int DM = TD ? TD : MAXD;
   constexpr int QM = TQ ? TQ : MAXQ;
   const int D3 = D * D * D, Q3 = Q * Q * Q;
   if (part && active)
   {
      const long long base = e * D3;
      for (int i = tx + Q * ty; i < D3; i += Q * Q)
      {
         bufA[i] = GATHER ? gather_value(x, gmap, mask, base + i) : x[base + i];
      }
   }
   __syncthreads();

   // per-thread copies of row qx of B and G
   T rBx[DM], rGx[DM];
#pragma unroll
   for (int d = 0; d < DM; ++d)
   {
      if (d < D && part) { rBx[d] = sB[tx * D + d]; rGx[d] = sG[tx * D + d]; }
   }

   // stage 1 (x): BX[dz][dy][qx] = sum_dx X[dz][dy][dx] B[qx][dx], GX with G
   T *BX = bufB, *GX = bufB + D * D * Q;
   for (int dy = ty; part && dy < D; dy += Q)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         T u = 0, v = 0;
         const T *xr = bufA + D * (dy + D * dz);
#pragma unroll
         for (int dx = 0; dx < DM; ++dx)
         {
            if (dx >= D) { break; }
            const T xv = xr[dx];
            u += xv * rBx[dx];
            v += xv * rGx[dx];
         }
         BX[(dz * D + dy) * Q + tx] = u;
         GX[(dz * D + dy) * Q + tx] = v;
      }
   }
   __syncthreads();

   T oA[DM], oB[DM], oC[DM];
#pragma unroll
   for (int dz = 0; dz < DM; ++dz) { oA[dz] = 0; oB[dz] = 0; oC[dz] = 0; }
   if (part)
   {
      // stage 2 (y) into registers: rA = G_x B_y, rBv = B_x G_y, rC = B_x B_y
      T rA[DM], rBv[DM], rC[DM];
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         T a = 0, b = 0, c = 0;
#pragma unroll
         for (int dy = 0; dy < DM; ++dy)
         {
            if (dy >= D) { break; }
            const T bx = BX[(dz * D + dy) * Q + tx];
            const T gx = GX[(dz * D + dy) * Q + tx];
            const T by = sB[ty * D + dy], gy = sG[ty * D + dy];
            a += gx * by;
            b += bx * gy;
            c += bx * by;
         }
         rA[dz] = a; rBv[dz] = b; rC[dz] = c;
      }

      // stage 3 (z) + pointwise qdata + backward z, fused per qz
      const T *qe = qd + e * (symm ? 6 : 9) * Q3 + tx + Q * ty;
#pragma unroll
      for (int qz = 0; qz < QM; ++qz)
      {
         if (qz >= Q) { break; }
         T gx = 0, gy = 0, gz = 0;
#pragma unroll
         for (int dz = 0; dz < DM; ++dz)
         {
            if (dz >= D) { break; }
            const T bz = sB[qz * D + dz], gzv = sG[qz * D + dz];
            gx += bz * rA[dz];
            gy += bz * rBv[dz];
            gz += gzv * rC[dz];
         }
         T ox = 0, oy = 0, oz = 0;
         if (active)
         {
            const T *qp = qe + Q * Q * qz;
            if (symm)
            {
               const T O11 = __ldg(qp), O12 = __ldg(qp + Q3), O13 = __ldg(qp + 2 * Q3);
               const T O22 = __ldg(qp + 3 * Q3), O23 = __ldg(qp + 4 * Q3);
               const T O33 = __ldg(qp + 5 * Q3);
               ox = O11 * gx + O12 * gy + O13 * gz;
               oy = O12 * gx + O22 * gy + O23 * gz;
               oz = O13 * gx + O23 * gy + O33 * gz;
            }
            else
            {
               const T O11 = __ldg(qp), O12 = __ldg(qp + Q3), O13 = __ldg(qp + 2 * Q3);
               const T O21 = __ldg(qp + 3 * Q3), O22 = __ldg(qp + 4 * Q3);
               const T O23 = __ldg(qp + 5 * Q3), O31 = __ldg(qp + 6 * Q3);
               const T O32 = __ldg(qp + 7 * Q3), O33 = __ldg(qp + 8 * Q3);
               ox = O11 * gx + O12 * gy + O13 * gz;
               oy = O21 * gx + O22 * gy + O23 * gz;
               oz = O31 * gx + O32 * gy + O33 * gz;
            }
         }
#pragma unroll
         for (int dz = 0; dz < DM; ++dz)
         {
            if (dz >= D) { break; }
            const T bz = sB[qz * D + dz], gzv = sG[qz * D + dz];
            oA[dz] += bz * ox;
            oB[dz] += bz * oy;
            oC[dz] += gzv * oz;
         }
      }
   }
   // T0|T1|T2 [dz][qy][qx] in bufA (X is dead: every thread passed the
   // barrier after stage 1, and stage 2 reads only bufB)
   T *T0 = bufA, *T1 = bufA + D * Q * Q, *T2 = bufA + 2 * D * Q * Q;
   if (part)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         T0[(dz * Q + ty) * Q + tx] = oA[dz];
         T1[(dz * Q + ty) * Q + tx] = oB[dz];
         T2[(dz * Q + ty) * Q + tx] = oC[dz];
      }
   }
   __syncthreads();

   // stage 2^T (y): thread (qx, dy): U0 = sum_qy T0 B[qy][dy],
   // U12 = sum_qy T1 G[qy][dy] + T2 B[qy][dy]  (into bufB)
   T *U0 = bufB, *U12 = bufB + D * D * Q;
   for (int dy = ty; part && dy < D; dy += Q)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         T a = 0, b = 0;
#pragma unroll
         for (int qy = 0; qy < QM; ++qy)
         {
            if (qy >= Q) { break; }
            const T by = sB[qy * D + dy], gy = sG[qy * D + dy];
            const int o = (dz * Q + qy) * Q + tx;
            a += T0[o] * by;
            b += T1[o] * gy + T2[o] * by;
         }
         U0[(dz * D + dy) * Q + tx] = a;
         U12[(dz * D + dy) * Q + tx] = b;
      }
   }
   __syncthreads();

   // stage 1^T (x): thread (dx, dy): y = sum_qx G[qx][dx] U0 + B[qx][dx] U12
   if (part && active)
   {
      const long long base = e * D3;
      for (int dy = ty; dy < D; dy += Q)
      {
         for (int dx = tx; dx < D; dx += Q)
         {
#pragma unroll
            for (int dz = 0; dz < DM; ++dz)
            {
               if (dz >= D) { break; }
               T v = 0;
#pragma unroll
               for (int qx = 0; qx < QM; ++qx)
               {
                  if (qx >= Q) { break; }
                  const int o = (dz * D + dy) * Q + qx;
                  v += sG[qx * D + dx] * U0[o] + sB[qx * D + dx] * U12[o];
               }
               const long long k = base + dx + D * (dy + D * dz);
               y[k] = accumulate ? y[k] + v : v;
            }
         }
      }
   }
}

template <typename T, int TD, int TQ, bool GATHER>
__global__ void diffusion_apply_kernel(int ne, int symm, int d1d, int q1d,
                                       const T *__restrict__ gB,
                                       const T *__restrict__ gG,
                                       const T *__restrict__ qd,
                                       const T *__restrict__ x,
                                       const int *__restrict__ gmap,
                                       const unsigned char *__restrict__ mask,
                                       T *__restrict__ y, int accumulate,
                                       const int *__restrict__ skip)
{
   if (skip && *skip) { return; }   // uniform per launch: solver finished
   const int D = TD ? TD : d1d;
   const int Q = TQ ? TQ : q1d;
   const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
   const int e = blockIdx.x * blockDim.z + tz;

   extern __shared__ __align__(16) unsigned char smem_raw[];
   T *sB = reinterpret_cast<T *>(smem_raw);       // [Q][D]
   T *sG = sB + Q * D;                            // [Q][D]
   const int per = diff_smem_per_elem(D, Q);
   T *bufA = sG + Q * D + tz * per;               // X, then T0|T1|T2
   T *bufB = bufA + (per - 2 * D * D * Q);        // BX|GX, then U0|U12
   const int tid = tx + Q * (ty + Q * tz);
   const int nthr = Q * Q * blockDim.z;
   for (int i = tid; i < Q * D; i += nthr)
   {
      const int q = i % Q, d = i / Q;
      sB[q * D + d] = gB[i];
      sG[q * D + d] = gG[i];
   }
   diffusion_element<T, TD, TQ, GATHER>(e, e < ne, true, D, Q, tx, ty, symm, sB, sG, bufA, bufB,
                                        qd, x, gmap, mask, y, accumulate);
}

template <typename T, int TD, int TQ, bool GATHER>
__global__ void mass_apply_kernel(int ne, int d1d, int q1d,
                                  const T *__restrict__ gB,
                                  const T *__restrict__ qd,
                                  const T *__restrict__ x,
                                  const int *__restrict__ gmap,
                                  const unsigned char *__restrict__ mask,
                                  T *__restrict__ y, int accumulate,
                                  const int *__restrict__ skip)
{
   if (skip && *skip) { return; }
   constexpr int DM = TD ? TD : GBPA_MAX_1D;
   constexpr int QM = TQ ? TQ : GBPA_MAX_1D;
   const int D = TD ? TD : d1d;
   const int Q = TQ ? TQ : q1d;
   const int D3 = D * D * D, Q3 = Q * Q * Q;
   const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
   const int e = blockIdx.x * blockDim.z + tz;
   const bool active = e < ne;

   extern __shared__ __align__(16) unsigned char smem_raw[];
   T *sB = reinterpret_cast<T *>(smem_raw);
   const int per = mass_smem_per_elem(D, Q);
   T *bufA = sB + Q * D + tz * per;
   T *bufB = bufA + (per - D * D * Q);

   const int tid = tx + Q * (ty + Q * tz);
   const int nthr = Q * Q * blockDim.z;
   for (int i = tid; i < Q * D; i += nthr) { sB[(i % Q) * D + i / Q] = gB[i]; }
   if (active)
   {
      const long long base = (long long)e * D3;
      for (int i = tx + Q * ty; i < D3; i += Q * Q)
      {
         bufA[i] = GATHER ? gather_value(x, gmap, mask, base + i) : x[base + i];
      }
   }
   __syncthreads();
   T rBx[DM];
#pragma unroll
   for (int d = 0; d < DM; ++d) { if (d < D) { rBx[d] = sB[tx * D + d]; } }
   T *BX = bufB;
   for (int dy = ty; dy < D; dy += Q)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         T u = 0;
         const T *xr = bufA + D * (dy + D * dz);
#pragma unroll
         for (int dx = 0; dx < DM; ++dx) { if (dx >= D) { break; } u += xr[dx] * rBx[dx]; }
         BX[(dz * D + dy) * Q + tx] = u;
      }
   }
   __syncthreads();
   T r[DM];
#pragma unroll
   for (int dz = 0; dz < DM; ++dz)
   {
      if (dz >= D) { break; }
      T a = 0;
#pragma unroll
      for (int dy = 0; dy < DM; ++dy)
      {
         if (dy >= D) { break; }
         a += BX[(dz * D + dy) * Q + tx] * sB[ty * D + dy];
      }
      r[dz] = a;
   }
   T o[DM];
#pragma unroll
   for (int dz = 0; dz < DM; ++dz) { o[dz] = 0; }
   const T *qe = qd + (long long)e * Q3 + tx + Q * ty;
#pragma unroll
   for (int qz = 0; qz < QM; ++qz)
   {
      if (qz >= Q) { break; }
      T v = 0;
#pragma unroll
      for (int dz = 0; dz < DM; ++dz) { if (dz >= D) { break; } v += sB[qz * D + dz] * r[dz]; }
      v = active ? v * __ldg(qe + Q * Q * qz) : T(0);
#pragma unroll
      for (int dz = 0; dz < DM; ++dz) { if (dz >= D) { break; } o[dz] += sB[qz * D + dz] * v; }
   }
   T *T0 = bufA;
#pragma unroll
   for (int dz = 0; dz < DM; ++dz) { if (dz >= D) { break; } T0[(dz * Q + ty) * Q + tx] = o[dz]; }
   __syncthreads();
   T *U = bufB;
   for (int dy = ty; dy < D; dy += Q)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         T a = 0;
#pragma unroll
         for (int qy = 0; qy < QM; ++qy)
         {
            if (qy >= Q) { break; }
            a += T0[(dz * Q + qy) * Q + tx] * sB[qy * D + dy];
         }
         U[(dz * D + dy) * Q + tx] = a;
      }
   }
   __syncthreads();
   if (active)
   {
      const long long base = (long long)e * D3;
      for (int dy = ty; dy < D; dy += Q)
         for (int dx = tx; dx < D; dx += Q)
         {
#pragma unroll
            for (int dz = 0; dz < DM; ++dz)
            {
               if (dz >= D) { break; }
               T v = 0;
#pragma unroll
               for (int qx = 0; qx < QM; ++qx)
               {
                  if (qx >= Q) { break; }
                  v += sB[qx * D + dx] * U[(dz * D + dy) * Q + qx];
               }
               const long long k = base + dx + D * (dy + D * dz);
               y[k] = accumulate ? y[k] + v : v;
            }
         }
   }
}

} // namespace gbpa
