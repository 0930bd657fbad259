// Shared pieces of the tensor-core (tcgen05) apply kernels: inline-PTX
// wrappers for the shared-memory matrix descriptors, the MMA and its commit,
// TMEM loads and stores, fences, mbarrier transaction counts and bulk copies,
// the fp16 hi/lo limb split, and the host-side Kronecker table builder.
//
// Shared-memory operands use the no-swizzle canonical layouts: 8 x 8 fp16
// core matrices of 128 contiguous bytes. K-major: core (row group rg, k group
// kg) at byte (kg * rows/8 + rg) * 128, LBO = rows/8 * 128 between
// K-adjacent cores, SBO = 128 between row groups. The backward GEMMs read a
// forward table chunk as MN-major (N = dofs contiguous in each 16-byte row):
// LBO = 128 between K-adjacent cores (chunk columns), SBO = NC/8 * 128
// between N-adjacent cores.
#pragma once
#include "gbpa_apply_kernels.cuh"
#include <cuda_fp16.h>
#include <cmath>
#include <vector>

namespace gbpa
{
namespace tc
{

__device__ __forceinline__ uint64_t smem_desc(unsigned saddr, unsigned lbo, unsigned sbo)
{
   uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
   d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
   d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
   d |= (uint64_t)1 << 46;   // descriptor version of sm_100-family tensor cores
   return d;                 // base offset 0, no swizzle
}

// instruction descriptor, kind::f16: fp16 A (K-major) and B (K-major, or
// MN-major with b_mn), FP32 accumulate
__host__ __device__ constexpr uint32_t instr_desc(int M, int N, bool b_mn = false)
{
   return (1u << 4) | (b_mn ? (1u << 16) : 0u) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(unsigned dtmem, uint64_t da, uint64_t db, uint32_t idesc, bool acc)
{
   asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                ::"r"(dtmem), "l"(da), "l"(db), "r"(idesc), "r"((unsigned)acc) : "memory");
}
// A operand in tensor memory (lane = row, two fp16 per column along K)
__device__ __forceinline__ void mma_f16_ta(unsigned dtmem, unsigned atmem, uint64_t db, uint32_t idesc, bool acc)
{
   asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}"
                ::"r"(dtmem), "r"(atmem), "l"(db), "r"(idesc), "r"((unsigned)acc) : "memory");
}
__device__ __forceinline__ void mma_commit(unsigned long long *bar)
{
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                ::"r"(smem_u32(bar)) : "memory");
}
// one lane of a converged warp (the lane that issues single-thread
// tcgen05 instructions while the whole warp keeps their operands uniform)
__device__ __forceinline__ bool elect_one()
{
   unsigned pred = 0;
   asm volatile("{\n .reg .pred p;\n elect.sync _|p, 0xffffffff;\n selp.u32 %0, 1, 0, p;\n}" : "=r"(pred));
   return pred != 0;
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
// 8 / 4 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_st8(unsigned taddr, const unsigned *v)
{
   asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                ::"r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                : "memory");
}
__device__ __forceinline__ void tmem_st4(unsigned taddr, const unsigned *v)
{
   asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};"
                ::"r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]) : "memory");
}
// 4 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld4(unsigned taddr, float *v)
{
   unsigned r[4];
   asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                : "r"(taddr));
#pragma unroll
   for (int j = 0; j < 4; ++j) { v[j] = __uint_as_float(r[j]); }
}
// 2 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_st2(unsigned taddr, const unsigned *v)
{
   asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1,%2};" ::"r"(taddr), "r"(v[0]), "r"(v[1]) : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect(unsigned long long *bar, unsigned bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                : "memory");
}
// start bringing a global range into L2 (no completion to wait for)
__device__ __forceinline__ void bulk_prefetch_l2(const void *gsrc, unsigned bytes)
{
   asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(gsrc), "r"(bytes) : "memory");
}
// bring the line holding p into L2 (no completion, no register)
__device__ __forceinline__ void prefetch_l2(const void *p)
{
   asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
__device__ __forceinline__ void bulk_g2s(void *sdst, const void *gsrc, unsigned bytes, unsigned long long *bar)
{
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(smem_u32(sdst)), "l"(gsrc), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// (v0, v1) -> one 32-bit word of each fp16 limb, v0 in the low half:
// hi = fp16(v), lo = fp16(v - hi), both rounded to nearest even (one paired
// conversion per limb; the same bits as converting each value on its own)
__device__ __forceinline__ void split2(float v0, float v1, unsigned &hi, unsigned &lo)
{
   const __half2 h = __floats2half2_rn(v0, v1);
   const float2 hf = __half22float2(h);
   const __half2 l = __floats2half2_rn(v0 - hf.x, v1 - hf.y);
   hi = *reinterpret_cast<const unsigned *>(&h);
   lo = *reinterpret_cast<const unsigned *>(&l);
}

// v -> (hi, lo) fp16 limbs of 8 consecutive values, two per 32-bit word
// (the lower k in the low half): one 16-byte core-matrix row, or four TMEM
// columns of an A operand
__device__ __forceinline__ void split8(const float *v, uint4 &hi, uint4 &lo)
{
   split2(v[0], v[1], hi.x, lo.x);
   split2(v[2], v[3], hi.y, lo.y);
   split2(v[4], v[5], hi.z, lo.z);
   split2(v[6], v[7], hi.w, lo.w);
}

// v -> (hi, lo) fp16 limbs of 4 consecutive values, two per 32-bit word
__device__ __forceinline__ void split4(const float *v, unsigned *hi, unsigned *lo)
{
   split2(v[0], v[1], hi[0], lo[0]);
   split2(v[2], v[3], hi[1], lo[1]);
}

// Host: the Kronecker matrix of the 1D tables, K[3q+c][i] (row 3q+c, q = qx
// + Q(qy + Q qz); column i = dx + D(dy + D dz)): G B B, B G B, B B G for
// c = 0, 1, 2, from the (Q, D) column-major tables B, G. Rows are padded to
// nch chunks of nc = 3 PC rows, columns to kf (a multiple of 16). Each chunk is
// laid out as one fp16 limb pair (hi, then lo) of nc x kf K-major core
// matrices -- the forward GEMM's B operand, which the backward GEMM reads as
// MN-major. R = the largest absolute row sum of K (the bound the per-element
// output scale is chosen from).
inline void build_kron_tables(int D, int Q, int PC, const double *B, const double *G,
                              std::vector<unsigned char> &tf, double &R)
{
   const int D3 = D * D * D, Q3 = Q * Q * Q, NC = 3 * PC;
   const int KF = (D3 + 15) / 16 * 16;
   const int NCH = (Q3 + PC - 1) / PC;
   const int NR = NCH * NC;
   const size_t BF_LIMB = (size_t)NC * KF * 2;
   std::vector<double> K((size_t)NR * KF, 0.0);
   for (int q = 0; q < Q3; ++q)
   {
      const int qx = q % Q, qy = (q / Q) % Q, qz = q / (Q * Q);
      for (int i = 0; i < D3; ++i)
      {
         const int dx = i % D, dy = (i / D) % D, dz = i / (D * D);
         const double bx = B[qx + Q * dx], by = B[qy + Q * dy], bz = B[qz + Q * dz];
         const double gx = G[qx + Q * dx], gy = G[qy + Q * dy], gz = G[qz + Q * dz];
         K[(size_t)(3 * q + 0) * KF + i] = gx * by * bz;
         K[(size_t)(3 * q + 1) * KF + i] = bx * gy * bz;
         K[(size_t)(3 * q + 2) * KF + i] = bx * by * gz;
      }
   }
   R = 0.0;
   for (int n = 0; n < NR; ++n)
   {
      double s = 0.0;
      for (int i = 0; i < KF; ++i) { s += fabs(K[(size_t)n * KF + i]); }
      R = fmax(R, s);
   }
   tf.assign((size_t)NCH * 2 * BF_LIMB, 0);
   auto put = [](unsigned char *base, size_t byte, double v, int limb) {
      const __half h = __double2half(v);
      const __half l = __double2half(v - (double)__half2float(h));
      const unsigned short u = __half_as_ushort(limb ? l : h);
      base[byte] = (unsigned char)(u & 0xFF);
      base[byte + 1] = (unsigned char)(u >> 8);
   };
   for (int c = 0; c < NCH; ++c)
   {
      for (int j = 0; j < NC; ++j)
      {
         for (int i = 0; i < KF; ++i)
         {
            const double v = K[(size_t)(c * NC + j) * KF + i];
            for (int limb = 0; limb < 2; ++limb)
            {
               unsigned char *bf = tf.data() + (size_t)c * 2 * BF_LIMB + limb * BF_LIMB;
               put(bf, (size_t)((i / 8) * (NC / 8) + j / 8) * 128 + (j % 8) * 16 + (i % 8) * 2, v, limb);
            }
         }
      }
   }
}

} // namespace tc
} // namespace gbpa
