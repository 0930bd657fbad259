// Sum-factorised 3D diffusion and mass kernels, templated on an arithmetic
// (AR) and on compile-time (D, Q); TD = TQ = 0 selects the generic
// runtime-size variant.
//
// Thread layout ("2D slab"): block = (Q, Q, nbz); thread (tx, ty, tz) owns the
// quadrature column (qx = tx, qy = ty) of element blockIdx.x*nbz + tz and keeps
// the z-direction of every intermediate in registers. Only the x- and y-
// contractions exchange data through shared memory, so an element costs four
// block barriers. The contraction sequence is the reference's (x, y, z
// forward; pointwise 3x3 qdata; z, y, x backward; fem/integ/
// bilininteg_diffusion_kernels.hpp:989-1215), reorganised so the z-forward,
// pointwise and z-backward stages fuse into one register loop over qz.
//
// Arithmetics:
//   ArF64  native FP64 (the FP64 pipe: ~1.26 TFLOP/s on GB300)
//   ArF32  native FP32
//   ArX2   FP64-accurate "double-float": every value is an unevaluated sum
//          hi + lo of two floats; products use the exact FMA error term and
//          sums the exact two-sum error (Dekker 1971; Knuth TAOCP vol. 2,
//          4.2.2), so all arithmetic runs on the FP32 pipes (58x the FP64
//          rate on GB300) with ~2^-44 relative error per operation. Inputs and
//          outputs stay FP64; qdata is stored pre-split as float2 (hi, lo),
//          the same 8 bytes per entry as FP64.
#pragma once
#include "gbpa_internal.cuh"

namespace gbpa
{

struct f2
{
   float h, l;
};

struct ArF64
{
   using V = double; using In = double; using Qd = double;
   static __device__ __forceinline__ V zero() { return 0.0; }
   static __device__ __forceinline__ void mac(V &acc, V a, V b) { acc = fma(a, b, acc); }
   static __device__ __forceinline__ V in(In x) { return x; }
   static __device__ __forceinline__ V neg(V a) { return -a; }
   static __device__ __forceinline__ V fin(V a) { return a; }
   static __device__ __forceinline__ In out(V v) { return v; }
   static __device__ __forceinline__ V ldq(const Qd *p) { return __ldg(p); }
   static __device__ __forceinline__ V lds(const Qd *p) { return *p; }
   static constexpr bool kTmaQd = false;   // FP64-pipe bound: no staging
};

struct ArF32
{
   using V = float; using In = float; using Qd = float;
   static __device__ __forceinline__ V zero() { return 0.f; }
   static __device__ __forceinline__ void mac(V &acc, V a, V b) { acc = fmaf(a, b, acc); }
   static __device__ __forceinline__ V in(In x) { return x; }
   static __device__ __forceinline__ V neg(V a) { return -a; }
   static __device__ __forceinline__ V fin(V a) { return a; }
   static __device__ __forceinline__ In out(V v) { return v; }
   static __device__ __forceinline__ V ldq(const Qd *p) { return __ldg(p); }
   static __device__ __forceinline__ V lds(const Qd *p) { return *p; }
   // memory-latency bound: stage the block's qdata with one TMA bulk copy
   static constexpr bool kTmaQd = true;
};

struct ArX2
{
   using V = f2; using In = double; using Qd = float2;
   static __device__ __forceinline__ V zero() { return {0.f, 0.f}; }
   // acc += a * b. The rounded product p = a.h*b.h and its exact error
   // fma(a.h, b.h, -p) (plus the cross terms) form the addend; acc.h + p is
   // an exact two-sum whose error joins acc.l. acc.l is left unnormalised
   // until fin(). The _rn intrinsics keep the compiler from contracting the
   // rounded operations into FMAs, which would break the error terms.
   static __device__ __forceinline__ void mac(V &acc, V a, V b)
   {
      const float p = __fmul_rn(a.h, b.h);
      float e = __fmaf_rn(a.h, b.h, -p);
      e = __fmaf_rn(a.h, b.l, e);
      e = __fmaf_rn(a.l, b.h, e);
      const float s = __fadd_rn(acc.h, p);
      const float bb = __fadd_rn(s, -acc.h);
      const float err = __fadd_rn(__fadd_rn(acc.h, -__fadd_rn(s, -bb)), __fadd_rn(p, -bb));
      acc.l = __fadd_rn(acc.l, __fadd_rn(e, err));
      acc.h = s;
   }
   static __device__ __forceinline__ V in(In x)
   {
      const float h = __double2float_rn(x);
      return {h, __double2float_rn(x - (double)h)};
   }
   static __device__ __forceinline__ V neg(V a) { return {-a.h, -a.l}; }
   // renormalise (fast two-sum; |l| << |h|)
   static __device__ __forceinline__ V fin(V a)
   {
      const float s = __fadd_rn(a.h, a.l);
      return {s, __fadd_rn(a.l, -__fadd_rn(s, -a.h))};
   }
   static __device__ __forceinline__ In out(V v) { return (double)v.h + (double)v.l; }
   static __device__ __forceinline__ V ldq(const Qd *p)
   {
      const float2 t = __ldg(p);
      return {t.x, t.y};
   }
   static __device__ __forceinline__ V lds(const Qd *p)
   {
      const float2 t = *p;
      return {t.x, t.y};
   }
   static constexpr bool kTmaQd = false;
};

// COH: x was written earlier in the same launch by other blocks (persistent
// solvers), so it is read through L2 (__ldcg) instead of the non-coherent
// read-only path.
// ------------------------------------------------ TMA bulk copy + mbarrier
// A block's qdata (nbz consecutive elements) is one contiguous range, so one
// thread stages it into shared memory with a single cp.async.bulk that
// completes on an mbarrier; the other threads meanwhile gather x and run the
// x/y contractions. The source must start on a 16-byte boundary and the size
// be a multiple of 16 bytes (the host checks both).
__device__ __forceinline__ unsigned smem_u32(const void *p)
{
   return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void tma_load_1d(void *sdst, const void *gsrc, unsigned bytes,
                                            unsigned long long *bar)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(smem_u32(sdst)), "l"(gsrc), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
// Wait for phase `parity` of the mbarrier with a bounded number of polls.
// Returns false on expiry; the caller then writes NaN for its element, so a
// copy that never lands shows up as a non-finite result (PCG reports
// GBPA_ERR_NOT_FINITE) and the kernel always terminates.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity,
                                          long long max_polls = 1LL << 24)
{
   for (long long it = 0; it < max_polls; ++it)
   {
      unsigned ok;
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                   " selp.u32 %0, 1, 0, p;\n}"
                   : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
      if (ok) { return true; }
   }
   return false;
}

// Stage the qdata of elements [e0, e0 + cnt) (eb bytes each) into `tile` with
// one bulk copy of the enclosing 16-byte-aligned byte range of the array (the
// extra bytes on either side belong to neighbouring elements of the same
// array), completing on `bar`. Returns element e0's qdata inside the tile, or
// nullptr when the rounded range would end past the array (then the block
// reads global memory). The array base must be 16-byte aligned (the host
// checks). Called by every thread of the block; the decision is uniform.
template <typename Qd>
__device__ __forceinline__ Qd *stage_qdata(unsigned char *tile, unsigned long long *bar,
                                           const Qd *qd, int ne, int e0, int cnt, size_t eb,
                                           int tid)
{
   const size_t b0 = (size_t)e0 * eb, b1 = (size_t)(e0 + cnt) * eb, total = (size_t)ne * eb;
   const size_t a0 = b0 & ~size_t(15), a1 = (b1 + 15) & ~size_t(15);
   if (a1 > total) { return nullptr; }
   if (tid == 0) { mbar_init(bar, 1); }
   __syncthreads();
   if (tid == 0)
   {
      tma_load_1d(tile, reinterpret_cast<const unsigned char *>(qd) + a0, (unsigned)(a1 - a0), bar);
   }
   return reinterpret_cast<Qd *>(tile + (b0 - a0));
}

template <typename AR, bool COH = false>
__device__ __forceinline__ typename AR::V gather_value(const typename AR::In *__restrict__ x,
                                                       const int *__restrict__ gmap,
                                                       const unsigned char *__restrict__ mask,
                                                       long long slot, int xs = 1)
{
   const int g = __ldg(gmap + slot);
   if (g == GBPA_GATHER_SKIP) { return AR::zero(); }   // pre-masked map: constrained dof
   const int j = g >= 0 ? g : -1 - g;
   if (mask && __ldg(mask + j)) { return AR::zero(); }
   const typename AR::In *p = x + (long long)j * xs;
   const typename AR::V v = AR::in(COH ? __ldcg(p) : __ldg(p));
   return g >= 0 ? v : AR::neg(v);
}

// One E-slot's result r. mode 0: y[k] = r; 1: y[k] += r (E-vector y);
// GBPA_OUT_ATOMIC: r is added atomically, with the slot's sign, into the
// L-vector y at the dof the gather map gives the slot (ElementRestriction::
// MultTranspose fused into the apply, summed in arrival order instead of the
// CSR row order); constrained slots (GBPA_GATHER_SKIP, or masked dofs) add
// nothing.
template <typename T>
__device__ __forceinline__ void store_result(T *y, long long k, long long slot, T r, int mode,
                                             const int *__restrict__ gmap,
                                             const unsigned char *__restrict__ mask)
{
   if (mode == GBPA_OUT_ATOMIC)
   {
      const int g = __ldg(gmap + slot);
      if (g == GBPA_GATHER_SKIP) { return; }
      const int j = g >= 0 ? g : -1 - g;
      if (mask && __ldg(mask + j)) { return; }
      atomicAdd(y + j, g >= 0 ? r : -r);
   }
   else
   {
      y[k] = mode ? y[k] + r : r;
   }
}

// Shared memory (in V units) per element for the diffusion apply.
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
template <typename AR, int TD, int TQ, bool GATHER, int MAXD = GBPA_MAX_1D, int MAXQ = GBPA_MAX_1D,
          bool COH = false>
__device__ __forceinline__ void
diffusion_element(long long e, bool active, bool part, int D, int Q, int tx, int ty, int symm,
                  const typename AR::V *__restrict__ sB, const typename AR::V *__restrict__ sG,
                  typename AR::V *__restrict__ bufA, typename AR::V *__restrict__ bufB,
                  const typename AR::Qd *__restrict__ qd, const typename AR::In *__restrict__ x,
                  const int *__restrict__ gmap, const unsigned char *__restrict__ mask,
                  typename AR::In *__restrict__ y, int accumulate, int xs = 1, int ys = 1,
                  const typename AR::Qd *sQ = nullptr, unsigned long long *qbar = nullptr)
{
   // xs, ys: element strides of the gathered L-vector and of the output
   // E-vector (> 1 for right-hand sides stored interleaved).
   // sQ, qbar: this element's qdata staged in shared memory by a TMA bulk
   // copy completing on qbar (phase 0); nullptr reads qdata from global.
   using V = typename AR::V;
   constexpr int DM = TD ? TD : MAXD;
   constexpr int QM = TQ ? TQ : MAXQ;
   const int D3 = D * D * D, Q3 = Q * Q * Q;
   if constexpr (GATHER && TD > 0 && TQ > 0)
   {
      // compile-time sizes: all of the thread's map entries first, then all
      // of its dof loads, so the dependent map -> x loads overlap instead of
      // taking one round trip per dof
      constexpr int Q2 = TQ * TQ, NPT = (TD * TD * TD + Q2 - 1) / Q2;
      const int ts = tx + TQ * ty;
      const long long base = e * D3;
      int gi[NPT];
#pragma unroll
      for (int k = 0; k < NPT; ++k)
      {
         const int i = ts + k * Q2;
         gi[k] = (part && active && i < D3) ? __ldg(gmap + base + i) : GBPA_GATHER_SKIP;
      }
      V gv[NPT];
#pragma unroll
      for (int k = 0; k < NPT; ++k)
      {
         const int g = gi[k];
         V v = AR::zero();
         if (g != GBPA_GATHER_SKIP)
         {
            const int j = g >= 0 ? g : -1 - g;
            if (!(mask && __ldg(mask + j)))
            {
               const typename AR::In *p = x + (long long)j * xs;
               v = AR::in(COH ? __ldcg(p) : __ldg(p));
               if (g < 0) { v = AR::neg(v); }
            }
         }
         gv[k] = v;
      }
#pragma unroll
      for (int k = 0; k < NPT; ++k)
      {
         const int i = ts + k * Q2;
         if (part && active && i < D3) { bufA[i] = gv[k]; }
      }
   }
   else if (part && active)
   {
      const long long base = e * D3;
      for (int i = tx + Q * ty; i < D3; i += Q * Q)
      {
         bufA[i] = GATHER ? gather_value<AR, COH>(x, gmap, mask, base + i, xs)
                          : AR::in(x[(base + i) * xs]);
      }
   }
   __syncthreads();

   // per-thread copies of row qx of B and G
   V rBx[DM], rGx[DM];
#pragma unroll
   for (int d = 0; d < DM; ++d)
   {
      if (d < D && part) { rBx[d] = sB[tx * D + d]; rGx[d] = sG[tx * D + d]; }
   }

   // stage 1 (x): BX[dz][dy][qx] = sum_dx X[dz][dy][dx] B[qx][dx], GX with G
   V *BX = bufB, *GX = bufB + D * D * Q;
   for (int dy = ty; part && dy < D; dy += Q)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         V u = AR::zero(), v = AR::zero();
         const V *xr = bufA + D * (dy + D * dz);
#pragma unroll
         for (int dx = 0; dx < DM; ++dx)
         {
            if (dx >= D) { break; }
            const V xv = xr[dx];
            AR::mac(u, xv, rBx[dx]);
            AR::mac(v, xv, rGx[dx]);
         }
         BX[(dz * D + dy) * Q + tx] = AR::fin(u);
         GX[(dz * D + dy) * Q + tx] = AR::fin(v);
      }
   }
   __syncthreads();

   V oA[DM], oB[DM], oC[DM];
#pragma unroll
   for (int dz = 0; dz < DM; ++dz) { oA[dz] = AR::zero(); oB[dz] = AR::zero(); oC[dz] = AR::zero(); }
   bool qok = true;   // false if the staged qdata never arrived
   if (part)
   {
      // stage 2 (y) into registers: rA = G_x B_y, rBv = B_x G_y, rC = B_x B_y
      V rA[DM], rBv[DM], rC[DM];
      V rBy[DM], rGy[DM];   // row qy = ty of B and G, reused for every dz
#pragma unroll
      for (int dy = 0; dy < DM; ++dy)
      {
         if (dy < D) { rBy[dy] = sB[ty * D + dy]; rGy[dy] = sG[ty * D + dy]; }
      }
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         V a = AR::zero(), b = AR::zero(), c = AR::zero();
#pragma unroll
         for (int dy = 0; dy < DM; ++dy)
         {
            if (dy >= D) { break; }
            const V bx = BX[(dz * D + dy) * Q + tx];
            const V gx = GX[(dz * D + dy) * Q + tx];
            const V by = rBy[dy], gy = rGy[dy];
            AR::mac(a, gx, by);
            AR::mac(b, bx, gy);
            AR::mac(c, bx, by);
         }
         rA[dz] = AR::fin(a); rBv[dz] = AR::fin(b); rC[dz] = AR::fin(c);
      }

      // stage 3 (z) + pointwise qdata + backward z, fused per qz
      if (sQ && active) { qok = mbar_wait(qbar, 0); }
      const typename AR::Qd *qe = (sQ ? sQ : qd + e * (symm ? 6 : 9) * Q3) + tx + Q * ty;
      // staged qdata is read from shared memory; otherwise read-only global
      auto LQ = [sQ](const typename AR::Qd *p) { return sQ ? AR::lds(p) : AR::ldq(p); };
#pragma unroll
      for (int qz = 0; qz < QM; ++qz)
      {
         if (qz >= Q) { break; }
         V gx = AR::zero(), gy = AR::zero(), gz = AR::zero();
#pragma unroll
         for (int dz = 0; dz < DM; ++dz)
         {
            if (dz >= D) { break; }
            const V bz = sB[qz * D + dz], gzv = sG[qz * D + dz];
            AR::mac(gx, bz, rA[dz]);
            AR::mac(gy, bz, rBv[dz]);
            AR::mac(gz, gzv, rC[dz]);
         }
         gx = AR::fin(gx); gy = AR::fin(gy); gz = AR::fin(gz);
         V ox = AR::zero(), oy = AR::zero(), oz = AR::zero();
         if (active)
         {
            const typename AR::Qd *qp = qe + Q * Q * qz;
            if (symm)
            {
               const V O11 = LQ(qp), O12 = LQ(qp + Q3), O13 = LQ(qp + 2 * Q3);
               const V O22 = LQ(qp + 3 * Q3), O23 = LQ(qp + 4 * Q3), O33 = LQ(qp + 5 * Q3);
               AR::mac(ox, O11, gx); AR::mac(ox, O12, gy); AR::mac(ox, O13, gz);
               AR::mac(oy, O12, gx); AR::mac(oy, O22, gy); AR::mac(oy, O23, gz);
               AR::mac(oz, O13, gx); AR::mac(oz, O23, gy); AR::mac(oz, O33, gz);
            }
            else
            {
               const V O11 = LQ(qp), O12 = LQ(qp + Q3), O13 = LQ(qp + 2 * Q3);
               const V O21 = LQ(qp + 3 * Q3), O22 = LQ(qp + 4 * Q3);
               const V O23 = LQ(qp + 5 * Q3), O31 = LQ(qp + 6 * Q3);
               const V O32 = LQ(qp + 7 * Q3), O33 = LQ(qp + 8 * Q3);
               AR::mac(ox, O11, gx); AR::mac(ox, O12, gy); AR::mac(ox, O13, gz);
               AR::mac(oy, O21, gx); AR::mac(oy, O22, gy); AR::mac(oy, O23, gz);
               AR::mac(oz, O31, gx); AR::mac(oz, O32, gy); AR::mac(oz, O33, gz);
            }
            ox = AR::fin(ox); oy = AR::fin(oy); oz = AR::fin(oz);
         }
#pragma unroll
         for (int dz = 0; dz < DM; ++dz)
         {
            if (dz >= D) { break; }
            const V bz = sB[qz * D + dz], gzv = sG[qz * D + dz];
            AR::mac(oA[dz], bz, ox);
            AR::mac(oB[dz], bz, oy);
            AR::mac(oC[dz], gzv, oz);
         }
      }
   }
   // T0|T1|T2 [dz][qy][qx] in bufA (X is dead: every thread passed the
   // barrier after stage 1, and stage 2 reads only bufB)
   V *T0 = bufA, *T1 = bufA + D * Q * Q, *T2 = bufA + 2 * D * Q * Q;
   if (part)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         T0[(dz * Q + ty) * Q + tx] = AR::fin(oA[dz]);
         T1[(dz * Q + ty) * Q + tx] = AR::fin(oB[dz]);
         T2[(dz * Q + ty) * Q + tx] = AR::fin(oC[dz]);
      }
   }
   __syncthreads();

   // stage 2^T (y): thread (qx, dy): U0 = sum_qy T0 B[qy][dy],
   // U12 = sum_qy T1 G[qy][dy] + T2 B[qy][dy]  (into bufB)
   V *U0 = bufB, *U12 = bufB + D * D * Q;
   for (int dy = ty; part && dy < D; dy += Q)
   {
      V cBy[QM], cGy[QM];   // column dy of B and G, reused for every dz
#pragma unroll
      for (int qy = 0; qy < QM; ++qy)
      {
         if (qy < Q) { cBy[qy] = sB[qy * D + dy]; cGy[qy] = sG[qy * D + dy]; }
      }
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         V a = AR::zero(), b = AR::zero();
#pragma unroll
         for (int qy = 0; qy < QM; ++qy)
         {
            if (qy >= Q) { break; }
            const V by = cBy[qy], gy = cGy[qy];
            const int o = (dz * Q + qy) * Q + tx;
            AR::mac(a, T0[o], by);
            AR::mac(b, T1[o], gy);
            AR::mac(b, T2[o], by);
         }
         U0[(dz * D + dy) * Q + tx] = AR::fin(a);
         U12[(dz * D + dy) * Q + tx] = AR::fin(b);
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
            V cBx[QM], cGx[QM];   // column dx of B and G, reused for every dz
#pragma unroll
            for (int qx = 0; qx < QM; ++qx)
            {
               if (qx < Q) { cBx[qx] = sB[qx * D + dx]; cGx[qx] = sG[qx * D + dx]; }
            }
#pragma unroll
            for (int dz = 0; dz < DM; ++dz)
            {
               if (dz >= D) { break; }
               V v = AR::zero();
#pragma unroll
               for (int qx = 0; qx < QM; ++qx)
               {
                  if (qx >= Q) { break; }
                  const int o = (dz * D + dy) * Q + qx;
                  AR::mac(v, cGx[qx], U0[o]);
                  AR::mac(v, cBx[qx], U12[o]);
               }
               const long long slot = base + dx + D * (dy + D * dz);
               const typename AR::In r = qok ? AR::out(AR::fin(v)) : (typename AR::In)NAN;
               store_result(y, slot * ys, slot, r, accumulate, gmap, mask);
            }
         }
      }
   }
}

// One block's share of the diffusion apply: elements [e0, e0 + cnt) of an
// operator with ne elements (cnt <= blockDim.z), in the 2D-slab layout
// (Q, Q, nbz). Shared by the single-operator kernel and the batched kernel
// that maps blocks onto (problem, first element) pairs.
template <typename AR, int TD, int TQ, bool GATHER, int MAXD, int MAXQ>
__device__ __forceinline__ void diffusion_apply_slab(int ne, int e0, int cnt, int symm, int d1d,
                                                     int q1d, const typename AR::In *__restrict__ gB,
                                                     const typename AR::In *__restrict__ gG,
                                                     const typename AR::Qd *__restrict__ qd,
                                                     const typename AR::In *__restrict__ x,
                                                     const int *__restrict__ gmap,
                                                     const unsigned char *__restrict__ mask,
                                                     typename AR::In *__restrict__ y, int accumulate,
                                                     int tma)
{
   using V = typename AR::V;
   using Qd = typename AR::Qd;
   const int D = TD ? TD : d1d;
   const int Q = TQ ? TQ : q1d;
   const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
   const int nbz = blockDim.z;
   const int e = e0 + tz;

   extern __shared__ __align__(16) unsigned char smem_raw[];
   V *sB = reinterpret_cast<V *>(smem_raw);       // [Q][D]
   V *sG = sB + Q * D;                            // [Q][D]
   const int per = diff_smem_per_elem(D, Q);
   V *bufA = sG + Q * D + tz * per;               // X, then T0|T1|T2
   V *bufB = bufA + (per - 2 * D * D * Q);        // BX|GX, then U0|U12
   const int tid = tx + Q * (ty + Q * tz);
   const int nthr = Q * Q * nbz;
   // optional TMA staging of the block's qdata: [tile | mbarrier] after the buffers
   const int S = symm ? 6 : 9;
   const int Q3 = Q * Q * Q;
   Qd *sQ = nullptr;
   unsigned long long *bar = nullptr;
   if (AR::kTmaQd && tma)
   {
      const size_t eb = sizeof(Qd) * (size_t)S * Q3;
      size_t off = sizeof(V) * (2 * Q * D + (size_t)nbz * per);
      off = (off + 15) & ~size_t(15);
      unsigned char *tile = smem_raw + off;
      off += eb * nbz + 32;
      off = (off + 7) & ~size_t(7);
      bar = reinterpret_cast<unsigned long long *>(smem_raw + off);
      sQ = stage_qdata<Qd>(tile, bar, qd, ne, e0, cnt, eb, tid);
   }
   for (int i = tid; i < Q * D; i += nthr)
   {
      const int q = i % Q, d = i / Q;
      sB[q * D + d] = AR::in(gB[i]);
      sG[q * D + d] = AR::in(gG[i]);
   }
   diffusion_element<AR, TD, TQ, GATHER, MAXD, MAXQ>(e, tz < cnt, true, D, Q, tx, ty, symm, sB, sG,
                                                     bufA, bufB, qd, x, gmap, mask, y, accumulate,
                                                     1, 1, sQ ? sQ + (size_t)tz * S * Q3 : nullptr,
                                                     bar);
}

template <typename AR, int TD, int TQ, bool GATHER, int MAXD = GBPA_MAX_1D, int MAXQ = GBPA_MAX_1D>
__global__ void diffusion_apply_kernel(int ne, int symm, int d1d, int q1d,
                                       const typename AR::In *__restrict__ gB,
                                       const typename AR::In *__restrict__ gG,
                                       const typename AR::Qd *__restrict__ qd,
                                       const typename AR::In *__restrict__ x,
                                       const int *__restrict__ gmap,
                                       const unsigned char *__restrict__ mask,
                                       typename AR::In *__restrict__ y, int accumulate,
                                       const int *__restrict__ skip, int tma)
{
   if (skip && *skip) { return; }   // uniform per launch: solver finished
   const int e0 = blockIdx.x * blockDim.z;
   diffusion_apply_slab<AR, TD, TQ, GATHER, MAXD, MAXQ>(ne, e0, min((int)blockDim.z, ne - e0), symm,
                                                        d1d, q1d, gB, gG, qd, x, gmap, mask, y,
                                                        accumulate, tma);
}

// R right-hand sides stored interleaved (x[j*R + r], E-vector out
// y[(e*D^3 + k)*R + r]). Same layout as the single-vector kernel, block
// (Q, Q, nbz); each slab applies its element to the R vectors in turn. The
// block's qdata is staged once in shared memory (TMA bulk copy, when the
// 16-byte rules hold) and reused for all R vectors, so HBM delivers it once
// per R applies; otherwise the R passes re-read it through L1/L2.
template <typename AR, int TD, int TQ, int TR = 0>
__global__ void diffusion_apply_block_kernel(int ne, int nrhs_rt, int symm, int d1d, int q1d,
                                             const typename AR::In *__restrict__ gB,
                                             const typename AR::In *__restrict__ gG,
                                             const typename AR::Qd *__restrict__ qd,
                                             const typename AR::In *__restrict__ x,
                                             const int *__restrict__ gmap,
                                             const unsigned char *__restrict__ mask,
                                             typename AR::In *__restrict__ y,
                                             const int *__restrict__ skip, int tma)
{
   using V = typename AR::V;
   using Qd = typename AR::Qd;
   if (skip && *skip) { return; }
   const int nrhs = TR ? TR : nrhs_rt;   // TR > 0: the count (and strides) known at compile time
   const int D = TD ? TD : d1d;
   const int Q = TQ ? TQ : q1d;
   const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
   const int nbz = blockDim.z;
   const int e0 = blockIdx.x * nbz;
   const int e = e0 + tz;
   extern __shared__ __align__(16) unsigned char smem_raw[];
   V *sB = reinterpret_cast<V *>(smem_raw);
   V *sG = sB + Q * D;
   const int per = diff_smem_per_elem(D, Q);
   V *bufA = sG + Q * D + tz * per;
   V *bufB = bufA + (per - 2 * D * D * Q);
   const int tid = tx + Q * (ty + Q * tz);
   const int nthr = Q * Q * nbz;
   const int S = symm ? 6 : 9;
   const int Q3 = Q * Q * Q;
   Qd *sQ = nullptr;
   unsigned long long *bar = nullptr;
   if (tma)
   {
      const size_t eb = sizeof(Qd) * (size_t)S * Q3;
      size_t off = sizeof(V) * (2 * Q * D + (size_t)nbz * per);
      off = (off + 15) & ~size_t(15);
      unsigned char *tile = smem_raw + off;
      off += eb * nbz + 32;
      off = (off + 7) & ~size_t(7);
      bar = reinterpret_cast<unsigned long long *>(smem_raw + off);
      sQ = stage_qdata<Qd>(tile, bar, qd, ne, e0, min(nbz, ne - e0), eb, tid);
   }
   for (int i = tid; i < Q * D; i += nthr)
   {
      const int q = i % Q, d = i / Q;
      sB[q * D + d] = AR::in(gB[i]);
      sG[q * D + d] = AR::in(gG[i]);
   }
   for (int r = 0; r < nrhs; ++r)
   {
      if (r > 0) { __syncthreads(); }   // previous pass done with this slab's buffers
      diffusion_element<AR, TD, TQ, true>(e, e < ne, true, D, Q, tx, ty, symm, sB, sG, bufA, bufB,
                                          qd, x + r, gmap, mask, y + r, 0, nrhs, nrhs,
                                          sQ ? sQ + (size_t)tz * S * Q3 : nullptr, bar);
   }
}

// 3D layout: block (Q, Q, Q * nbz), one thread per quadrature point (qx, qy,
// qz) of element blockIdx.x * nbz + threadIdx.z / Q. Every contraction goes
// through shared memory (six barriers per element); in the stages whose
// index runs over D < Q the threads beyond D idle. Same contraction sequence
// and arithmetic as the 2D slab; qdata is read fully coalesced (one point per
// thread). Per element two buffers are reused stage to stage:
//   buf1: X (D^3) -> A, Bv, C [dz][qy][qx] -> T0, T1, T2 [dz][qy][qx]
//   buf2: BX, GX [dz][dy][qx] -> O0, O1, O2 [qz][qy][qx] -> U0, U12 [dz][dy][qx]
template <int D, int Q>
__host__ __device__ constexpr int diff3d_buf1() { return D * D * D > 3 * D * Q * Q ? D * D * D : 3 * D * Q * Q; }
template <int D, int Q>
__host__ __device__ constexpr int diff3d_buf2() { return 2 * D * D * Q > 3 * Q * Q * Q ? 2 * D * D * Q : 3 * Q * Q * Q; }

// One block's share in the 3D layout: elements [e0, e0 + cnt) (cnt <=
// blockDim.z / Q) of an operator; shared by the single-operator kernel and the
// batched grouped apply.
template <typename AR, int D, int Q>
__device__ __forceinline__ void diffusion_3d_block(long long e0, int cnt, int symm,
                                                   const typename AR::In *__restrict__ gB,
                                                   const typename AR::In *__restrict__ gG,
                                                   const typename AR::Qd *__restrict__ qd,
                                                   const typename AR::In *__restrict__ x,
                                                   const int *__restrict__ gmap,
                                                   const unsigned char *__restrict__ mask,
                                                   typename AR::In *__restrict__ y, int mode)
{
   using V = typename AR::V;
   constexpr int D3 = D * D * D, Q3 = Q * Q * Q, DQQ = D * Q * Q, DDQ = D * D * Q;
   constexpr int S1 = diff3d_buf1<D, Q>(), S2 = diff3d_buf2<D, Q>();
   const int tx = threadIdx.x, ty = threadIdx.y;
   const int tz = threadIdx.z % Q, ez = threadIdx.z / Q;
   const long long e = e0 + ez;
   const bool active = ez < cnt;
   extern __shared__ __align__(16) unsigned char smem_raw[];
   V *sB = reinterpret_cast<V *>(smem_raw);   // [Q][D]
   V *sG = sB + Q * D;
   V *buf1 = sG + Q * D + (size_t)ez * (S1 + S2);
   V *buf2 = buf1 + S1;
   const int tid = tx + Q * (ty + Q * threadIdx.z);
   for (int i = tid; i < Q * D; i += Q * Q * blockDim.z)
   {
      const int q = i % Q, d = i / Q;
      sB[q * D + d] = AR::in(gB[i]);
      sG[q * D + d] = AR::in(gG[i]);
   }
   // gather: the element's thread t loads E-slot t (Q >= D, so Q^3 >= D^3)
   const int t = tx + Q * (ty + Q * tz);
   if (t < D3) { buf1[t] = active ? gather_value<AR>(x, gmap, mask, e * D3 + t) : AR::zero(); }
   __syncthreads();
   // stage 1 (x), thread (qx, dy, dz): BX, GX
   if (ty < D && tz < D)
   {
      V u = AR::zero(), v = AR::zero();
      const V *xr = buf1 + D * (ty + D * tz);
#pragma unroll
      for (int dx = 0; dx < D; ++dx)
      {
         const V xv = xr[dx];
         AR::mac(u, xv, sB[tx * D + dx]);
         AR::mac(v, xv, sG[tx * D + dx]);
      }
      const int o = (tz * D + ty) * Q + tx;
      buf2[o] = AR::fin(u);
      buf2[DDQ + o] = AR::fin(v);
   }
   __syncthreads();
   // stage 2 (y), thread (qx, qy, dz): A = G_x B_y, Bv = B_x G_y, C = B_x B_y
   if (tz < D)
   {
      V a = AR::zero(), b = AR::zero(), c = AR::zero();
#pragma unroll
      for (int dy = 0; dy < D; ++dy)
      {
         const int o = (tz * D + dy) * Q + tx;
         const V bx = buf2[o], gx = buf2[DDQ + o];
         const V by = sB[ty * D + dy], gy = sG[ty * D + dy];
         AR::mac(a, gx, by);
         AR::mac(b, bx, gy);
         AR::mac(c, bx, by);
      }
      const int o = (tz * Q + ty) * Q + tx;
      buf1[o] = AR::fin(a);
      buf1[DQQ + o] = AR::fin(b);
      buf1[2 * DQQ + o] = AR::fin(c);
   }
   __syncthreads();
   // stage 3 (z) and the pointwise 3x3 qdata product, thread (qx, qy, qz)
   {
      V gx = AR::zero(), gy = AR::zero(), gz = AR::zero();
#pragma unroll
      for (int dz = 0; dz < D; ++dz)
      {
         const int o = (dz * Q + ty) * Q + tx;
         const V bz = sB[tz * D + dz], gzv = sG[tz * D + dz];
         AR::mac(gx, bz, buf1[o]);
         AR::mac(gy, bz, buf1[DQQ + o]);
         AR::mac(gz, gzv, buf1[2 * DQQ + o]);
      }
      gx = AR::fin(gx); gy = AR::fin(gy); gz = AR::fin(gz);
      V ox = AR::zero(), oy = AR::zero(), oz = AR::zero();
      if (active)
      {
         const typename AR::Qd *qp = qd + e * (symm ? 6 : 9) * Q3 + t;
         if (symm)
         {
            const V O11 = AR::ldq(qp), O12 = AR::ldq(qp + Q3), O13 = AR::ldq(qp + 2 * Q3);
            const V O22 = AR::ldq(qp + 3 * Q3), O23 = AR::ldq(qp + 4 * Q3), O33 = AR::ldq(qp + 5 * Q3);
            AR::mac(ox, O11, gx); AR::mac(ox, O12, gy); AR::mac(ox, O13, gz);
            AR::mac(oy, O12, gx); AR::mac(oy, O22, gy); AR::mac(oy, O23, gz);
            AR::mac(oz, O13, gx); AR::mac(oz, O23, gy); AR::mac(oz, O33, gz);
         }
         else
         {
            const V O11 = AR::ldq(qp), O12 = AR::ldq(qp + Q3), O13 = AR::ldq(qp + 2 * Q3);
            const V O21 = AR::ldq(qp + 3 * Q3), O22 = AR::ldq(qp + 4 * Q3);
            const V O23 = AR::ldq(qp + 5 * Q3), O31 = AR::ldq(qp + 6 * Q3);
            const V O32 = AR::ldq(qp + 7 * Q3), O33 = AR::ldq(qp + 8 * Q3);
            AR::mac(ox, O11, gx); AR::mac(ox, O12, gy); AR::mac(ox, O13, gz);
            AR::mac(oy, O21, gx); AR::mac(oy, O22, gy); AR::mac(oy, O23, gz);
            AR::mac(oz, O31, gx); AR::mac(oz, O32, gy); AR::mac(oz, O33, gz);
         }
      }
      const int o = (tz * Q + ty) * Q + tx;
      buf2[o] = AR::fin(ox);
      buf2[Q3 + o] = AR::fin(oy);
      buf2[2 * Q3 + o] = AR::fin(oz);
   }
   __syncthreads();
   // backward z, thread (qx, qy, dz): T0 = B_z O0, T1 = B_z O1, T2 = G_z O2
   if (tz < D)
   {
      V a = AR::zero(), b = AR::zero(), c = AR::zero();
#pragma unroll
      for (int qz = 0; qz < Q; ++qz)
      {
         const int o = (qz * Q + ty) * Q + tx;
         const V bz = sB[qz * D + tz], gzv = sG[qz * D + tz];
         AR::mac(a, bz, buf2[o]);
         AR::mac(b, bz, buf2[Q3 + o]);
         AR::mac(c, gzv, buf2[2 * Q3 + o]);
      }
      const int o = (tz * Q + ty) * Q + tx;
      buf1[o] = AR::fin(a);
      buf1[DQQ + o] = AR::fin(b);
      buf1[2 * DQQ + o] = AR::fin(c);
   }
   __syncthreads();
   // backward y, thread (qx, dy, dz): U0 = B_y T0, U12 = G_y T1 + B_y T2
   if (ty < D && tz < D)
   {
      V a = AR::zero(), b = AR::zero();
#pragma unroll
      for (int qy = 0; qy < Q; ++qy)
      {
         const int o = (tz * Q + qy) * Q + tx;
         const V by = sB[qy * D + ty], gy = sG[qy * D + ty];
         AR::mac(a, buf1[o], by);
         AR::mac(b, buf1[DQQ + o], gy);
         AR::mac(b, buf1[2 * DQQ + o], by);
      }
      const int o = (tz * D + ty) * Q + tx;
      buf2[o] = AR::fin(a);
      buf2[DDQ + o] = AR::fin(b);
   }
   __syncthreads();
   // backward x, thread (dx, dy, dz): y = G_x U0 + B_x U12
   if (active && tx < D && ty < D && tz < D)
   {
      V v = AR::zero();
#pragma unroll
      for (int qx = 0; qx < Q; ++qx)
      {
         const int o = (tz * D + ty) * Q + qx;
         AR::mac(v, sG[qx * D + tx], buf2[o]);
         AR::mac(v, sB[qx * D + tx], buf2[DDQ + o]);
      }
      const long long slot = e * D3 + tx + D * (ty + D * tz);
      store_result(y, slot, slot, AR::out(AR::fin(v)), mode, gmap, mask);
   }
}

template <typename AR, int D, int Q>
__global__ void __launch_bounds__(1024, 2)
diffusion_apply_3d_kernel(int ne, int symm, const typename AR::In *__restrict__ gB,
                          const typename AR::In *__restrict__ gG, const typename AR::Qd *__restrict__ qd,
                          const typename AR::In *__restrict__ x, const int *__restrict__ gmap,
                          const unsigned char *__restrict__ mask, typename AR::In *__restrict__ y, int mode,
                          const int *__restrict__ skip)
{
   if (skip && *skip) { return; }   // uniform per launch: solver finished
   const int nbz = blockDim.z / Q;
   const long long e0 = (long long)blockIdx.x * nbz;
   diffusion_3d_block<AR, D, Q>(e0, (int)min((long long)nbz, ne - e0), symm, gB, gG, qd, x, gmap, mask, y, mode);
}

// Mass apply in the 3D layout (block (Q, Q, Q * nbz), one thread per
// quadrature point, gather fused), the 2D slab's multiply-adds in the same
// order. Per element: buf1 X (D^3) -> BBX [dz][qy][qx] -> T [dz][qy][qx];
// buf2 BX [dz][dy][qx] -> W [qz][qy][qx] -> U [dz][dy][qx].
template <int D, int Q>
__host__ __device__ constexpr int mass3d_buf1() { return D * D * D > D * Q * Q ? D * D * D : D * Q * Q; }
template <int D, int Q>
__host__ __device__ constexpr int mass3d_buf2() { return D * D * Q > Q * Q * Q ? D * D * Q : Q * Q * Q; }

template <typename AR, int D, int Q>
__global__ void __launch_bounds__(1024, 2)
mass_apply_3d_kernel(int ne, const typename AR::In *__restrict__ gB, const typename AR::Qd *__restrict__ qd,
                     const typename AR::In *__restrict__ x, const int *__restrict__ gmap,
                     const unsigned char *__restrict__ mask, typename AR::In *__restrict__ y, int mode,
                     const int *__restrict__ skip)
{
   using V = typename AR::V;
   constexpr int D3 = D * D * D, Q3 = Q * Q * Q;
   constexpr int S1 = mass3d_buf1<D, Q>(), S2 = mass3d_buf2<D, Q>();
   if (skip && *skip) { return; }
   const int tx = threadIdx.x, ty = threadIdx.y;
   const int tz = threadIdx.z % Q, ez = threadIdx.z / Q;
   const int nbz = blockDim.z / Q;
   const long long e = (long long)blockIdx.x * nbz + ez;
   const bool active = e < ne;
   extern __shared__ __align__(16) unsigned char smem_raw[];
   V *sB = reinterpret_cast<V *>(smem_raw);   // [Q][D]
   V *buf1 = sB + Q * D + (size_t)ez * (S1 + S2);
   V *buf2 = buf1 + S1;
   const int tid = tx + Q * (ty + Q * threadIdx.z);
   for (int i = tid; i < Q * D; i += Q * Q * blockDim.z) { sB[(i % Q) * D + i / Q] = AR::in(gB[i]); }
   const int t = tx + Q * (ty + Q * tz);
   if (t < D3) { buf1[t] = active ? gather_value<AR>(x, gmap, mask, e * D3 + t) : AR::zero(); }
   __syncthreads();
   // x, thread (qx, dy, dz)
   if (ty < D && tz < D)
   {
      V u = AR::zero();
      const V *xr = buf1 + D * (ty + D * tz);
#pragma unroll
      for (int dx = 0; dx < D; ++dx) { AR::mac(u, xr[dx], sB[tx * D + dx]); }
      buf2[(tz * D + ty) * Q + tx] = AR::fin(u);
   }
   __syncthreads();
   // y, thread (qx, qy, dz)
   if (tz < D)
   {
      V a = AR::zero();
#pragma unroll
      for (int dy = 0; dy < D; ++dy) { AR::mac(a, buf2[(tz * D + dy) * Q + tx], sB[ty * D + dy]); }
      buf1[(tz * Q + ty) * Q + tx] = AR::fin(a);
   }
   __syncthreads();
   // z and the pointwise qdata product, thread (qx, qy, qz)
   {
      V v = AR::zero();
#pragma unroll
      for (int dz = 0; dz < D; ++dz) { AR::mac(v, sB[tz * D + dz], buf1[(dz * Q + ty) * Q + tx]); }
      V w = AR::zero();
      if (active) { AR::mac(w, AR::fin(v), AR::ldq(qd + e * Q3 + t)); }
      buf2[(tz * Q + ty) * Q + tx] = AR::fin(w);
   }
   __syncthreads();
   // backward z, thread (qx, qy, dz)
   if (tz < D)
   {
      V o = AR::zero();
#pragma unroll
      for (int qz = 0; qz < Q; ++qz) { AR::mac(o, sB[qz * D + tz], buf2[(qz * Q + ty) * Q + tx]); }
      buf1[(tz * Q + ty) * Q + tx] = AR::fin(o);
   }
   __syncthreads();
   // backward y, thread (qx, dy, dz)
   if (ty < D && tz < D)
   {
      V a = AR::zero();
#pragma unroll
      for (int qy = 0; qy < Q; ++qy) { AR::mac(a, buf1[(tz * Q + qy) * Q + tx], sB[qy * D + ty]); }
      buf2[(tz * D + ty) * Q + tx] = AR::fin(a);
   }
   __syncthreads();
   // backward x, thread (dx, dy, dz)
   if (active && tx < D && ty < D && tz < D)
   {
      V v = AR::zero();
#pragma unroll
      for (int qx = 0; qx < Q; ++qx) { AR::mac(v, sB[qx * D + tx], buf2[(tz * D + ty) * Q + qx]); }
      const long long slot = e * D3 + tx + D * (ty + D * tz);
      store_result(y, slot, slot, AR::out(AR::fin(v)), mode, gmap, mask);
   }
}

template <typename AR, int TD, int TQ, bool GATHER, int MAXD = GBPA_MAX_1D, int MAXQ = GBPA_MAX_1D>
__global__ void mass_apply_kernel(int ne, int d1d, int q1d,
                                  const typename AR::In *__restrict__ gB,
                                  const typename AR::Qd *__restrict__ qd,
                                  const typename AR::In *__restrict__ x,
                                  const int *__restrict__ gmap,
                                  const unsigned char *__restrict__ mask,
                                  typename AR::In *__restrict__ y, int accumulate,
                                  const int *__restrict__ skip, int qdiv)
{
   // qdiv > 1: element e reads the qdata of element e / qdiv (the components
   // of a vector space sharing one scalar coefficient's qdata)
   using V = typename AR::V;
   if (skip && *skip) { return; }
   constexpr int DM = TD ? TD : MAXD;
   constexpr int QM = TQ ? TQ : MAXQ;
   const int D = TD ? TD : d1d;
   const int Q = TQ ? TQ : q1d;
   const int D3 = D * D * D, Q3 = Q * Q * Q;
   const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
   const int e = blockIdx.x * blockDim.z + tz;
   const bool active = e < ne;

   extern __shared__ __align__(16) unsigned char smem_raw[];
   V *sB = reinterpret_cast<V *>(smem_raw);
   const int per = mass_smem_per_elem(D, Q);
   V *bufA = sB + Q * D + tz * per;
   V *bufB = bufA + (per - D * D * Q);

   const int tid = tx + Q * (ty + Q * tz);
   const int nthr = Q * Q * blockDim.z;
   for (int i = tid; i < Q * D; i += nthr) { sB[(i % Q) * D + i / Q] = AR::in(gB[i]); }
   if (active)
   {
      const long long base = (long long)e * D3;
      for (int i = tx + Q * ty; i < D3; i += Q * Q)
      {
         bufA[i] = GATHER ? gather_value<AR>(x, gmap, mask, base + i) : AR::in(x[base + i]);
      }
   }
   __syncthreads();
   V rBx[DM];
#pragma unroll
   for (int d = 0; d < DM; ++d) { if (d < D) { rBx[d] = sB[tx * D + d]; } }
   V *BX = bufB;
   for (int dy = ty; dy < D; dy += Q)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         V u = AR::zero();
         const V *xr = bufA + D * (dy + D * dz);
#pragma unroll
         for (int dx = 0; dx < DM; ++dx) { if (dx >= D) { break; } AR::mac(u, xr[dx], rBx[dx]); }
         BX[(dz * D + dy) * Q + tx] = AR::fin(u);
      }
   }
   __syncthreads();
   V r[DM];
#pragma unroll
   for (int dz = 0; dz < DM; ++dz)
   {
      if (dz >= D) { break; }
      V a = AR::zero();
#pragma unroll
      for (int dy = 0; dy < DM; ++dy)
      {
         if (dy >= D) { break; }
         AR::mac(a, BX[(dz * D + dy) * Q + tx], sB[ty * D + dy]);
      }
      r[dz] = AR::fin(a);
   }
   V o[DM];
#pragma unroll
   for (int dz = 0; dz < DM; ++dz) { o[dz] = AR::zero(); }
   const typename AR::Qd *qe = qd + (long long)(e / qdiv) * Q3 + tx + Q * ty;
#pragma unroll
   for (int qz = 0; qz < QM; ++qz)
   {
      if (qz >= Q) { break; }
      V v = AR::zero();
#pragma unroll
      for (int dz = 0; dz < DM; ++dz) { if (dz >= D) { break; } AR::mac(v, sB[qz * D + dz], r[dz]); }
      V w = AR::zero();
      if (active) { AR::mac(w, AR::fin(v), AR::ldq(qe + Q * Q * qz)); }
      w = AR::fin(w);
#pragma unroll
      for (int dz = 0; dz < DM; ++dz) { if (dz >= D) { break; } AR::mac(o[dz], sB[qz * D + dz], w); }
   }
   V *T0 = bufA;
#pragma unroll
   for (int dz = 0; dz < DM; ++dz) { if (dz >= D) { break; } T0[(dz * Q + ty) * Q + tx] = AR::fin(o[dz]); }
   __syncthreads();
   V *U = bufB;
   for (int dy = ty; dy < D; dy += Q)
   {
#pragma unroll
      for (int dz = 0; dz < DM; ++dz)
      {
         if (dz >= D) { break; }
         V a = AR::zero();
#pragma unroll
         for (int qy = 0; qy < QM; ++qy)
         {
            if (qy >= Q) { break; }
            AR::mac(a, T0[(dz * Q + qy) * Q + tx], sB[qy * D + dy]);
         }
         U[(dz * D + dy) * Q + tx] = AR::fin(a);
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
               V v = AR::zero();
#pragma unroll
               for (int qx = 0; qx < QM; ++qx)
               {
                  if (qx >= Q) { break; }
                  AR::mac(v, sB[qx * D + dx], U[(dz * D + dy) * Q + qx]);
               }
               const long long k = base + dx + D * (dy + D * dz);
               const typename AR::In rr = AR::out(AR::fin(v));
               store_result(y, k, k, rr, accumulate, gmap, mask);
            }
         }
   }
}

} // namespace gbpa
