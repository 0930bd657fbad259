// FP32 diffusion apply on the fifth-generation tensor cores (tcgen05).
//
// The sum-factorised contraction of the 2D-slab and 3D kernels is replaced by
// two dense GEMMs per tile of 128 elements, with the elements in the M
// dimension (one TMEM lane per element):
//   forward   Gq[e][3q+c] = sum_i X[e][i] K[3q+c][i]       (M=128, N=3 PC, K=D^3)
//   pointwise O[e][3q+c]  = sum_d Dq[e][q][c][d] Gq[e][3q+d] (CUDA cores, FP32)
//   backward  Y[e][i]     = sum_n O[e][n] K[n][i]           (M=128, N=D^3, K=3 PC)
// K is the Kronecker matrix of the 1D tables: row 3q+c, q = qx + Q(qy + Q qz),
// column i = dx + D(dy + D dz), K = G(qx,dx) B(qy,dy) B(qz,dz) for c = 0,
// B G B for c = 1, B B G for c = 2 (the gradient in reference coordinates at
// quadrature point q, fem/integ/bilininteg_diffusion_kernels.hpp:989-1215).
// The quadrature points are processed in chunks of PC points: each chunk's
// forward GEMM lands in TMEM, the CUDA cores apply the qdata and write the
// chunk's O columns to shared memory, and the backward GEMM accumulates the
// chunk into the TMEM result. The tables (K and its transpose, split and laid
// out for the tensor cores) are the same for every tile and stream from L2 by
// bulk copies.
//
// FP32 accuracy on 16-bit tensor cores: every operand is split into two fp16
// limbs, v = hi + lo with hi = fp16(v), lo = fp16(v - hi), and a product is
// hi*hi + hi*lo + lo*hi (the lo*lo term is below FP32 rounding), accumulated
// in FP32. fp16's exponent range is kept by a power-of-two scale per element:
// x by 2^(14 - e) (e: the exponent of the element's max |x|), the pointwise
// output by a factor chosen from a bound of the element's qdata (qscale, one
// float per element, computed at operator creation). Both scales are undone
// exactly in the output.
//
// Shared-memory operands use the K-major, no-swizzle canonical layout:
// 8 x 8 fp16 core matrices of 128 contiguous bytes, core (row group rg,
// k group kg) at byte (kg * rows/8 + rg) * 128 (LBO = rows/8 * 128 between
// K-adjacent cores, SBO = 128 between row groups).
#include "gbpa_apply_kernels.cuh"
#include "gbpa_dispatch.cuh"
#include "gbpa_tc.cuh"
#include <cuda_fp16.h>
#include <cmath>
#include <vector>

namespace gbpa
{
namespace tc
{

template <int D, int Q, int PC>
struct Shape
{
   static constexpr int D3 = D * D * D;
   static constexpr int KF = (D3 + 15) / 16 * 16;   // dofs, padded to the MMA K step
   static constexpr int Q3 = Q * Q * Q;
   static constexpr int NC = 3 * PC;                // chunk columns (points x 3 components)
   static constexpr int NCH = (Q3 + PC - 1) / PC;   // chunks
   static constexpr int M = 128;                    // elements per tile
   static constexpr int A_LIMB = M * KF * 2;        // bytes of one fp16 limb of the x tile
   static constexpr int BF_LIMB = NC * KF * 2;      // one limb of a forward table chunk
   static constexpr int BB_LIMB = KF * NC * 2;      // one limb of a backward table chunk
   static constexpr int AB_LIMB = M * NC * 2;       // one limb of the chunk's O columns
   static constexpr int OFF_AF = 0;
   static constexpr int OFF_BF = OFF_AF + 2 * A_LIMB;
   static constexpr int OFF_BB = OFF_BF + 2 * BF_LIMB;
   static constexpr int OFF_AB = OFF_BB + 2 * BB_LIMB;
   static constexpr int SMEM = OFF_AB + 2 * AB_LIMB;
   static constexpr int STG = D3 | 1;               // staging row stride (odd: no bank conflicts)
   static constexpr int OFF_STG = OFF_BB;           // staging reuses the chunk buffers
   static constexpr int TF = 0, TB = 128;           // TMEM columns of the two accumulators
   static_assert(KF <= 128 && NC <= 128 && NC % 16 == 0, "accumulators must fit 128 TMEM columns");
   static_assert(OFF_STG + M * STG * 4 <= SMEM, "staging must fit in the chunk buffers");
   static_assert(SMEM <= 220 * 1024, "shared memory");
};

__device__ __forceinline__ uint64_t smem_desc(unsigned saddr, unsigned lbo, unsigned sbo)
{
   uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
   d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
   d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
   d |= (uint64_t)1 << 46;   // descriptor version of sm_100-family tensor cores
   return d;                 // base offset 0, no swizzle
}

// instruction descriptor, kind::f16: fp16 A and B (K-major), FP32 accumulate
__host__ __device__ constexpr uint32_t instr_desc(int M, int N)
{
   return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(unsigned dtmem, uint64_t da, uint64_t db, uint32_t idesc, bool acc)
{
   asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                ::"r"(dtmem), "l"(da), "l"(db), "r"(idesc), "r"((unsigned)acc) : "memory");
}
__device__ __forceinline__ void mma_commit(unsigned long long *bar)
{
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 8 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld8(unsigned taddr, float *v)
{
   unsigned r[8];
   asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                  "=r"(r[7])
                : "r"(taddr));
#pragma unroll
   for (int j = 0; j < 8; ++j) { v[j] = __uint_as_float(r[j]); }
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect(unsigned long long *bar, unsigned bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *sdst, const void *gsrc, unsigned bytes, unsigned long long *bar)
{
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(smem_u32(sdst)), "l"(gsrc), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// v -> (hi, lo) fp16 limbs of 8 consecutive values, packed for one 16-byte
// row of a core matrix
__device__ __forceinline__ void split8(const float *v, uint4 &hi, uint4 &lo)
{
   unsigned h[4], l[4];
#pragma unroll
   for (int q = 0; q < 4; ++q)
   {
      const __half h0 = __float2half_rn(v[2 * q]), h1 = __float2half_rn(v[2 * q + 1]);
      const __half l0 = __float2half_rn(v[2 * q] - __half2float(h0));
      const __half l1 = __float2half_rn(v[2 * q + 1] - __half2float(h1));
      h[q] = (unsigned)__half_as_ushort(h0) | ((unsigned)__half_as_ushort(h1) << 16);
      l[q] = (unsigned)__half_as_ushort(l0) | ((unsigned)__half_as_ushort(l1) << 16);
   }
   hi = make_uint4(h[0], h[1], h[2], h[3]);
   lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// Persistent kernel: one 256-thread CTA per SM walks tiles of 128 elements.
// Thread t: element row r = 32 (warp % 4) + lane (its TMEM lane), half
// h = warp / 4 (the two halves share a row and split its columns). Thread 0
// issues the bulk copies and the MMAs. Every wait is bounded: on expiry the
// tile's outputs are NaN and GBPA_FLAG_TIMEOUT is raised, and the control flow
// (barriers) stays uniform.
template <int D, int Q, int PC>
__global__ void __launch_bounds__(256, 1)
diffusion_tc_kernel(int ne, const unsigned char *__restrict__ tab_f, const unsigned char *__restrict__ tab_b,
                    const float *__restrict__ qd, const float *__restrict__ qscale, const float *__restrict__ x,
                    const int *__restrict__ gmap, const unsigned char *__restrict__ mask, float *__restrict__ y,
                    int mode, const int *__restrict__ skip, int *flags)
{
   using S = Shape<D, Q, PC>;
   if (skip && *skip) { return; }   // uniform per launch: the solver has finished
   extern __shared__ __align__(1024) unsigned char smem[];
   __shared__ __align__(8) unsigned long long bar_load, bar_mma;
   __shared__ unsigned tmem_base;
   __shared__ float s_max[2][128];
   __shared__ float s_sx[128], s_so[128];
   __shared__ int s_fail;
   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int half = warp >> 2;
   const int r = 32 * (warp & 3) + lane;
   const unsigned sbase = smem_u32(smem);
   float *stg = reinterpret_cast<float *>(smem + S::OFF_STG);

   if (tid == 0)
   {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_load)) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_mma)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      s_fail = 0;
   }
   if (warp == 0)
   {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;"
                   ::"r"(smem_u32(&tmem_base)) : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
   }
   fence_before();
   __syncthreads();
   fence_after();
   const unsigned tmem = tmem_base;
   const unsigned lane_off = (unsigned)(32 * (warp & 3)) << 16;
   // bounded wait; after a first expiry no later wait blocks (the kernel
   // then runs to its end quickly, writing NaN)
   volatile int *fail = &s_fail;
   auto wait = [&](unsigned long long *bar, unsigned ph) {
      if (*fail) { return; }
      if (!mbar_wait(bar, ph, 1LL << 20)) { *fail = 1; }
   };
   unsigned ph_load = 0, ph_mma = 0;
   constexpr uint32_t ID_F = instr_desc(128, S::NC), ID_B = instr_desc(128, S::KF);
   constexpr unsigned LBO_A = 16 * 128, LBO_BF = S::NC / 8 * 128, LBO_BB = S::KF / 8 * 128;
   const int ntiles = (ne + 127) / 128;

   for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
   {
      const long long e0 = (long long)tile * 128;
      // ---- gather the tile's x (ElementRestriction::Mult, signed map) into staging
      for (int s = tid; s < 128 * S::D3; s += 256)
      {
         const int el = s / S::D3, i = s - el * S::D3;
         const long long e = e0 + el;
         float v = 0.f;
         if (e < ne)
         {
            const int g = __ldg(gmap + e * S::D3 + i);
            if (g != GBPA_GATHER_SKIP)
            {
               const int j = g >= 0 ? g : -1 - g;
               if (!(mask && __ldg(mask + j)))
               {
                  v = __ldg(x + j);
                  if (g < 0) { v = -v; }
               }
            }
         }
         stg[el * S::STG + i] = v;
      }
      __syncthreads();
      {
         constexpr int H = (S::D3 + 1) / 2;
         float m = 0.f;
         for (int i = half * H; i < (half + 1) * H && i < S::D3; ++i) { m = fmaxf(m, fabsf(stg[r * S::STG + i])); }
         s_max[half][r] = m;
      }
      __syncthreads();
      if (half == 0)
      {
         const float m = fmaxf(s_max[0][r], s_max[1][r]);
         float sx = 1.f;
         if (m > 0.f && m <= 3.0e38f)
         {
            int ex;
            frexpf(m, &ex);                 // m < 2^ex
            sx = ldexpf(1.f, 14 - ex);      // m * sx in [2^13, 2^14)
         }
         s_sx[r] = sx;
         s_so[r] = e0 + r < ne ? __ldg(qscale + e0 + r) : 1.f;
      }
      __syncthreads();
      {
         const float sx = s_sx[r];
         for (int kg = half * (S::KF / 16); kg < (half + 1) * (S::KF / 16); ++kg)
         {
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
            {
               const int k = 8 * kg + j;
               v[j] = k < S::D3 ? stg[r * S::STG + k] * sx : 0.f;
            }
            uint4 hi, lo;
            split8(v, hi, lo);
            const int off = (kg * 16 + (r >> 3)) * 128 + (r & 7) * 16;
            *reinterpret_cast<uint4 *>(smem + S::OFF_AF + off) = hi;
            *reinterpret_cast<uint4 *>(smem + S::OFF_AF + S::A_LIMB + off) = lo;
         }
      }
      fence_async_smem();
      __syncthreads();

      const long long e = e0 + r;
      const bool act = e < ne;
      const float sx = s_sx[r], so = s_so[r];
      const float f = so / sx;   // exact: both are powers of two
      for (int c = 0; c < S::NCH; ++c)
      {
         if (tid == 0)
         {
            mbar_expect(&bar_load, 2 * S::BF_LIMB + 2 * S::BB_LIMB);
            bulk_g2s(smem + S::OFF_BF, tab_f + (size_t)c * 2 * S::BF_LIMB, 2 * S::BF_LIMB, &bar_load);
            bulk_g2s(smem + S::OFF_BB, tab_b + (size_t)c * 2 * S::BB_LIMB, 2 * S::BB_LIMB, &bar_load);
            wait(&bar_load, ph_load);
            fence_after();
            // forward: Gq = X K^T over the KF dofs, three limb products
#pragma unroll 1
            for (int s = 0; s < S::KF / 16; ++s)
            {
               const unsigned a0 = sbase + S::OFF_AF + s * 2 * LBO_A;
               const unsigned b0 = sbase + S::OFF_BF + s * 2 * LBO_BF;
               const uint64_t ahi = smem_desc(a0, LBO_A, 128), alo = smem_desc(a0 + S::A_LIMB, LBO_A, 128);
               const uint64_t bhi = smem_desc(b0, LBO_BF, 128), blo = smem_desc(b0 + S::BF_LIMB, LBO_BF, 128);
               mma_f16(tmem + S::TF, ahi, bhi, ID_F, s > 0);
               mma_f16(tmem + S::TF, ahi, blo, ID_F, true);
               mma_f16(tmem + S::TF, alo, bhi, ID_F, true);
            }
            mma_commit(&bar_mma);
         }
         ph_load ^= 1;
         wait(&bar_mma, ph_mma);
         ph_mma ^= 1;
         fence_after();
         // pointwise: this thread's PC/2 points of the chunk
         constexpr int NP = PC / 2, NV = 3 * NP;
         float gq[NV], o[NV];
#pragma unroll
         for (int j = 0; j < NV; j += 8)
         {
            tmem_ld8(tmem + lane_off + S::TF + half * NV + j, gq + j);
         }
         tmem_wait_ld();
#pragma unroll
         for (int p = 0; p < NP; ++p)
         {
            const int q = c * PC + half * NP + p;
            float O11 = 0.f, O12 = 0.f, O13 = 0.f, O22 = 0.f, O23 = 0.f, O33 = 0.f;
            if (act && q < S::Q3)
            {
               const float *qe = qd + e * 6 * S::Q3 + q;
               O11 = __ldg(qe); O12 = __ldg(qe + S::Q3); O13 = __ldg(qe + 2 * S::Q3);
               O22 = __ldg(qe + 3 * S::Q3); O23 = __ldg(qe + 4 * S::Q3); O33 = __ldg(qe + 5 * S::Q3);
            }
            const float gx = gq[3 * p], gy = gq[3 * p + 1], gz = gq[3 * p + 2];
            o[3 * p] = (O11 * gx + O12 * gy + O13 * gz) * f;
            o[3 * p + 1] = (O12 * gx + O22 * gy + O23 * gz) * f;
            o[3 * p + 2] = (O13 * gx + O23 * gy + O33 * gz) * f;
         }
#pragma unroll
         for (int jg = 0; jg < NV / 8; ++jg)
         {
            uint4 hi, lo;
            split8(o + 8 * jg, hi, lo);
            const int kg = half * (NV / 8) + jg;
            const int off = (kg * 16 + (r >> 3)) * 128 + (r & 7) * 16;
            *reinterpret_cast<uint4 *>(smem + S::OFF_AB + off) = hi;
            *reinterpret_cast<uint4 *>(smem + S::OFF_AB + S::AB_LIMB + off) = lo;
         }
         fence_async_smem();
         fence_before();
         __syncthreads();
         if (tid == 0)
         {
            fence_after();
            // backward: Y += O K over the chunk's columns
#pragma unroll 1
            for (int s = 0; s < S::NC / 16; ++s)
            {
               const unsigned a0 = sbase + S::OFF_AB + s * 2 * LBO_A;
               const unsigned b0 = sbase + S::OFF_BB + s * 2 * LBO_BB;
               const uint64_t ahi = smem_desc(a0, LBO_A, 128), alo = smem_desc(a0 + S::AB_LIMB, LBO_A, 128);
               const uint64_t bhi = smem_desc(b0, LBO_BB, 128), blo = smem_desc(b0 + S::BB_LIMB, LBO_BB, 128);
               mma_f16(tmem + S::TB, ahi, bhi, ID_B, c > 0 || s > 0);
               mma_f16(tmem + S::TB, ahi, blo, ID_B, true);
               mma_f16(tmem + S::TB, alo, bhi, ID_B, true);
            }
            mma_commit(&bar_mma);
         }
         wait(&bar_mma, ph_mma);
         ph_mma ^= 1;
         fence_after();
      }
      // ---- result: undo the output scale (the x scale was undone in the
      // pointwise factor f), stage, store the tile contiguously
      {
         const float inv = 1.f / so;
         constexpr int NH = S::KF / 2;
#pragma unroll
         for (int j = 0; j < NH; j += 8)
         {
            float v[8];
            tmem_ld8(tmem + lane_off + S::TB + half * NH + j, v);
            tmem_wait_ld();
#pragma unroll
            for (int k = 0; k < 8; ++k)
            {
               const int i = half * NH + j + k;
               if (i < S::D3) { stg[r * S::STG + i] = v[k] * inv; }
            }
         }
      }
      fence_before();
      __syncthreads();
      const bool failed = s_fail != 0;
      for (int s = tid; s < 128 * S::D3; s += 256)
      {
         const int el = s / S::D3, i = s - el * S::D3;
         const long long ee = e0 + el;
         if (ee >= ne) { continue; }
         const float v = failed ? NAN : stg[el * S::STG + i];
         const long long slot = ee * S::D3 + i;
         store_result(y, slot, slot, v, mode, gmap, mask);
      }
      __syncthreads();
   }
   if (tid == 0 && s_fail) { atomicOr(flags, GBPA_FLAG_TIMEOUT); }
   fence_before();
   __syncthreads();
   if (warp == 0)
   {
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
   }
}

// ------------------------------------------------------------- host side
template <int D, int Q, int PC>
static void build_tables_t(const double *B, const double *G, std::vector<unsigned char> &tf,
                           std::vector<unsigned char> &tb, double &R)
{
   using S = Shape<D, Q, PC>;
   const int NR = S::NCH * S::NC;                  // Kronecker rows, padded to whole chunks
   std::vector<double> K((size_t)NR * S::KF, 0.0);
   for (int q = 0; q < S::Q3; ++q)
   {
      const int qx = q % Q, qy = (q / Q) % Q, qz = q / (Q * Q);
      for (int i = 0; i < S::D3; ++i)
      {
         const int dx = i % D, dy = (i / D) % D, dz = i / (D * D);
         // (Q, D) column-major tables
         const double bx = B[qx + Q * dx], by = B[qy + Q * dy], bz = B[qz + Q * dz];
         const double gx = G[qx + Q * dx], gy = G[qy + Q * dy], gz = G[qz + Q * dz];
         K[(size_t)(3 * q + 0) * S::KF + i] = gx * by * bz;
         K[(size_t)(3 * q + 1) * S::KF + i] = bx * gy * bz;
         K[(size_t)(3 * q + 2) * S::KF + i] = bx * by * gz;
      }
   }
   R = 0.0;
   for (int n = 0; n < NR; ++n)
   {
      double s = 0.0;
      for (int i = 0; i < S::KF; ++i) { s += fabs(K[(size_t)n * S::KF + i]); }
      R = fmax(R, s);
   }
   tf.assign((size_t)S::NCH * 2 * S::BF_LIMB, 0);
   tb.assign((size_t)S::NCH * 2 * S::BB_LIMB, 0);
   auto put = [](unsigned char *base, size_t byte, double v, int limb) {
      const __half h = __double2half(v);
      const __half l = __double2half(v - (double)__half2float(h));
      const unsigned short u = __half_as_ushort(limb ? l : h);
      base[byte] = (unsigned char)(u & 0xFF);
      base[byte + 1] = (unsigned char)(u >> 8);
   };
   for (int c = 0; c < S::NCH; ++c)
   {
      for (int j = 0; j < S::NC; ++j)
      {
         for (int i = 0; i < S::KF; ++i)
         {
            const double v = K[(size_t)(c * S::NC + j) * S::KF + i];
            for (int limb = 0; limb < 2; ++limb)
            {
               // forward chunk: rows j (N), K = i
               unsigned char *bf = tf.data() + (size_t)c * 2 * S::BF_LIMB + limb * S::BF_LIMB;
               put(bf, (size_t)((i / 8) * (S::NC / 8) + j / 8) * 128 + (j % 8) * 16 + (i % 8) * 2, v, limb);
               // backward chunk: rows i (N), K = j
               unsigned char *bb = tb.data() + (size_t)c * 2 * S::BB_LIMB + limb * S::BB_LIMB;
               put(bb, (size_t)((j / 8) * (S::KF / 8) + i / 8) * 128 + (i % 8) * 16 + (j % 8) * 2, v, limb);
            }
         }
      }
   }
}

#define GBPA_TC_LIST(X) X(3, 4, 32) X(4, 5, 32) X(5, 6, 32)

bool supported(int D, int Q)
{
#define GBPA_CASE(d, q, pc) if (D == d && Q == q) { return true; }
   GBPA_TC_LIST(GBPA_CASE)
#undef GBPA_CASE
   return false;
}

int build_tables(int D, int Q, const double *B, const double *G, Tables *t)
{
   std::vector<unsigned char> tf, tb;
   double R = 0.0;
   bool found = false;
#define GBPA_CASE(d, q, pc) \
   if (D == d && Q == q) { build_tables_t<d, q, pc>(B, G, tf, tb, R); found = true; }
   GBPA_TC_LIST(GBPA_CASE)
#undef GBPA_CASE
   if (!found) { return GBPA_ERR_UNSUPPORTED; }
   t->D = D; t->Q = Q; t->R = R;
   int rc = check_cuda(cudaMalloc(&t->fwd, tf.size()), "cudaMalloc(tc tables)");
   if (!rc) { rc = check_cuda(cudaMalloc(&t->bwd, tb.size()), "cudaMalloc(tc tables)"); }
   if (!rc) { rc = check_cuda(cudaMemcpy(t->fwd, tf.data(), tf.size(), cudaMemcpyHostToDevice), "copy tc tables"); }
   if (!rc) { rc = check_cuda(cudaMemcpy(t->bwd, tb.data(), tb.size(), cudaMemcpyHostToDevice), "copy tc tables"); }
   if (rc) { free_tables(t); }
   return rc;
}

void free_tables(Tables *t)
{
   cudaFree(t->fwd); cudaFree(t->bwd);
   t->fwd = t->bwd = nullptr;
}

// qscale[e] = 2^-ceil(log2(qmax_e R)), qmax_e the largest absolute row sum of
// the element's symmetric 3x3 qdata blocks: |O * qscale| <= 2^14 whenever the
// scaled x has |x| < 2^14.
__global__ void qscale_kernel(int ne, int Q3, const float *__restrict__ qd, float R, float *__restrict__ qs)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x)
   {
      const float *p = qd + (long long)e * 6 * Q3;
      float m = 0.f;
      for (int q = 0; q < Q3; ++q)
      {
         const float a = fabsf(p[q]), b = fabsf(p[q + Q3]), c = fabsf(p[q + 2 * Q3]);
         const float d = fabsf(p[q + 3 * Q3]), f = fabsf(p[q + 4 * Q3]), g = fabsf(p[q + 5 * Q3]);
         m = fmaxf(m, fmaxf(a + b + c, fmaxf(b + d + f, c + f + g)));
      }
      const float bound = m * R;
      float s = 1.f;
      if (bound > 0.f && bound <= 3.0e38f)
      {
         int ex;
         frexpf(bound, &ex);   // bound < 2^ex
         s = ldexpf(1.f, -ex);
      }
      qs[e] = s;
   }
}

int launch_qscale(gbpa_ctx *ctx, int ne, int Q, const float *qd, float R, float *qscale)
{
   if (ne <= 0) { return GBPA_SUCCESS; }
   qscale_kernel<<<grid_for(ne, 256), 256, 0, ctx->stream>>>(ne, Q * Q * Q, qd, R, qscale);
   return last_launch(ctx, "tc_qscale");
}

template <int D, int Q, int PC>
static int launch_t(gbpa_ctx *ctx, int ne, const Tables &t, const float *qd, const float *qscale, const float *x,
                    const int *gmap, const unsigned char *mask, float *y, int mode, const int *skip)
{
   using S = Shape<D, Q, PC>;
   const void *k = (const void *)diffusion_tc_kernel<D, Q, PC>;
   const int ntiles = (ne + 127) / 128;
   const int grid = std::min(ntiles, ctx->num_sms > 0 ? ctx->num_sms : 148);
   const unsigned char *tf = t.fwd, *tb = t.bwd;
   int *flags = ctx->d_flags;
   void *args[] = {&ne, (void *)&tf, (void *)&tb, (void *)&qd, (void *)&qscale, (void *)&x, (void *)&gmap,
                   (void *)&mask, &y, &mode, (void *)&skip, &flags};
   return launch_generic(ctx, k, dim3(grid), dim3(256), args, S::SMEM, "diffusion_tc");
}

int launch_diffusion_f32(gbpa_ctx *ctx, int ne, int D, int Q, const Tables &t, const float *qd,
                         const float *qscale, const float *x, const int *gmap, const unsigned char *mask,
                         float *y, int mode, const int *skip)
{
   if (ne == 0) { return GBPA_SUCCESS; }
   if (t.D != D || t.Q != Q || !t.fwd || !gmap) { return GBPA_ERR_UNSUPPORTED; }
#define GBPA_CASE(d, q, pc) \
   if (D == d && Q == q) { return launch_t<d, q, pc>(ctx, ne, t, qd, qscale, x, gmap, mask, y, mode, skip); }
   GBPA_TC_LIST(GBPA_CASE)
#undef GBPA_CASE
   return GBPA_ERR_UNSUPPORTED;
}

} // namespace tc
} // namespace gbpa
