// Block (several right-hand sides) FP32 diffusion apply on the tensor cores.
//
// The element contraction is the Kronecker-GEMM form of the single tensor-core
// kernel (gbpa_apply_tc.cu): forward Gq = X K^T, pointwise O = Dq Gq on the
// CUDA cores, backward Y = O K, the quadrature points in chunks of PC. Here
// the 128 GEMM rows of a tile are EL = 128 / R elements times R right-hand
// sides (row r: element r / R, right-hand side r % R), so every element's
// qdata and gather map serve R rows: one tile reads the qdata of 16 elements
// for 8 vectors. Vectors are stored interleaved, x[j R + r]; the output is the
// block E-vector y[(e D^3 + i) R + r] (the layout of the CUDA-core block
// apply, fem/bilinearform_ext.cpp:487-564 applied to R vectors at once).
//
// Operands (D^3 up to 216, K = D^3 padded to 16):
//   x tile     hi limb in TMEM (the A operand of the hi*hi and hi*lo
//              products), lo limb in shared memory (A of lo*hi)
//   O chunk    fp16 limbs in TMEM (the backward GEMM's A operand)
//   tables     a ring of three chunks in shared memory (bulk copies from L2):
//              a chunk's copy starts once the backward GEMM of the chunk
//              three back has released its buffer, a chunk ahead of its use
//   result     TMEM (KF columns); at the start of a tile the same columns
//              hold the gathered raw x until its row maximum is known
// The output goes from TMEM straight to the block E-vector (the R vectors
// of a dof are adjacent: a warp writes whole 32-byte sectors).
//
// FP32 accuracy as in the single kernel: fp16 hi/lo limbs, three products,
// FP32 accumulation, a power-of-two scale per row for x and per element for
// the pointwise output, both undone exactly in the output.
#include "gbpa_apply_kernels.cuh"
#include "gbpa_dispatch.cuh"
#include "gbpa_tc.cuh"
#include "gbpa_tc_ptx.cuh"
#include <algorithm>

namespace gbpa
{
namespace tc
{

// Timeline probes for kernel development: compiled in only with
// -DGBPA_TC_TRACE (SM clock of CTA 0's first tiles into a device table).
#ifdef GBPA_TC_TRACE
__device__ unsigned long long g_tcb_trace[2048];
#define TCB_TRACE(it, i)                                                           \
   do                                                                              \
   {                                                                               \
      if (blockIdx.x == 0 && (it) < 2) { g_tcb_trace[(it) * 1024 + (i)] = clock64(); } \
   } while (0)
#else
#define TCB_TRACE(it, i) do { } while (0)
#endif

template <int D, int Q, int PC, int R>
struct BShape
{
   static constexpr int D3 = D * D * D;
   static constexpr int KF = (D3 + 15) / 16 * 16;   // dofs, padded to the MMA K step
   static constexpr int PARTS = 4;                  // epilogue threads per GEMM row
   static constexpr int EPI = 128 * PARTS;          // epilogue threads (16 warps)
   static constexpr int KH = KF / PARTS;            // dofs per part of a row
   static constexpr int Q3 = Q * Q * Q;
   static constexpr int NC = 3 * PC;                // chunk columns
   static constexpr int NCH = (Q3 + PC - 1) / PC;   // chunks
   static constexpr int NP = PC / PARTS;            // points of a chunk per thread
   static constexpr int NV = 3 * NP;                // chunk columns per thread
   static constexpr int NQ = 6 * NP;                // qdata values per thread and chunk
   static constexpr int M = 128;                    // GEMM rows per tile
   static constexpr int EL = M / R;                 // elements per tile
   static constexpr int XL_BYTES = M * KF * 2;      // the x tile's lo limb
   static constexpr int BF_LIMB = NC * KF * 2;      // one limb of a table chunk
   static constexpr int NT = 3;                     // table ring depth
   static constexpr int QD_BYTES = PARTS * NQ * EL * 4; // one tile-chunk of qdata, [part][k][element]
   static constexpr int QT_CHUNK = PARTS * NQ * EL; // its floats
   static constexpr int OFF_XL = 0;
   static constexpr int OFF_T = OFF_XL + XL_BYTES;
   static constexpr int OFF_QD = OFF_T + NT * 2 * BF_LIMB;
   static constexpr int SMEM = OFF_QD + 2 * QD_BYTES;
   // tensor memory: the result (and the raw x at a tile's start), two forward
   // accumulators, the x tile's hi limb and the chunk's O limbs (two values
   // per column)
   static constexpr int TB = 0, TF0 = 224, TF1 = 272, TXH = 320, TOH = TXH + KF / 2, TOL = TOH + NC / 2;
   static __device__ __forceinline__ int off_t(int c) { return OFF_T + (c % NT) * 2 * BF_LIMB; }
   static_assert(M % R == 0 && R <= 32 && 32 % R == 0, "rows of one element stay in one warp");
   static_assert(KF <= TF0 && TF0 + NC <= TF1 && TF1 + NC <= TXH && TOL + NC / 2 <= 512, "TMEM columns");
   static_assert(KF <= 256 && NC <= 64 && NC % 16 == 0 && NV == 12 && KH % 8 == 0, "MMA shapes");
   static_assert(NCH % 2 == 0 && NCH >= NT, "the chunk loop is unrolled by two");
   static_assert(SMEM <= 222 * 1024, "shared memory");
   static_assert(QD_BYTES % 16 == 0 && BF_LIMB % 16 == 0, "bulk copy sizes");
   static_assert((EL * D3 * 4) % 16 == 0, "a full tile's map rows are whole 16-byte units");
   static_assert(KH / 8 <= NCH, "the next tile's x is prefetched over the chunk loop");
};

// Persistent kernel: one CTA per SM walks tiles of EL elements x R vectors.
// Warps 0-15 gather, split, apply the qdata and store (thread: row r = 32
// (warp % 4) + lane, part warp / 4 -- a quarter -- of the row's columns);
// warp 16 issues the MMAs (one elected lane), lane 0 of warp 17 the bulk
// copies (table chunks into
// a ring of three, qdata chunks into two buffers, each refilled once the chunk
// it held is released). A barrier that could complete twice before one of
// its waiters looks is kept per buffer (tfree, dfree, fwd, qd, qfree), so
// every parity wait sees each phase. Every wait is bounded:
// after a first expiry no wait blocks, no further MMA or copy is started,
// the outputs are NaN and GBPA_FLAG_TIMEOUT is raised; the MMA warp and the
// copy producer wait (bounded) for their work in flight before the CTA
// releases TMEM and exits.
template <int D, int Q, int PC, int R>
__global__ void __launch_bounds__(576, 1)
diffusion_tc_block_kernel(int ne, const unsigned char *__restrict__ tab_f, const float *__restrict__ qT,
                          const float *__restrict__ qscale, const float *__restrict__ x,
                          const int *__restrict__ gmap, const unsigned char *__restrict__ mask,
                          float *__restrict__ y, const int *__restrict__ skip, int *flags)
{
   using S = BShape<D, Q, PC, R>;
   if (skip && *skip) { return; }
   extern __shared__ __align__(1024) unsigned char smem[];
   // mbarriers: table ring 0-2, qdata 0-1 (bulk copies); af, ab, dfree0/1,
   // qfree0/1 (one arrival per epilogue thread); fwd0/1, bwd, tfree0-2, drain (MMA
   // commits)
   constexpr int NMB = 18;
   __shared__ __align__(8) unsigned long long mb[NMB];
   __shared__ unsigned tmem_base;
   __shared__ float s_max[4][128];
   __shared__ int s_fail;
   unsigned long long *MB_T = mb, *MB_QD = mb + 3, *MB_AF = mb + 5, *MB_AB = mb + 6, *MB_DFREE = mb + 7;
   unsigned long long *MB_QFREE = mb + 9, *MB_FWD = mb + 11, *MB_BWD = mb + 13, *MB_TFREE = mb + 14;
   unsigned long long *MB_DRAIN = mb + 17;
   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int part = (warp >> 2) & 3;   // epilogue warps 0-15: the part of the row's columns
   const int r = 32 * (warp & 3) + lane;
   const unsigned sbase = smem_u32(smem);

   if (tid == 0)
   {
      const unsigned E = S::EPI;
      const unsigned counts[NMB] = {1, 1, 1, 1, 1, E, E, E, E, E, E, 1, 1, 1, 1, 1, 1, 1};
      for (int i = 0; i < NMB; ++i)
      {
         asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mb + i)), "r"(counts[i]) : "memory");
      }
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      s_fail = 0;
   }
   if (warp == 0)
   {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;"
                   ::"r"(smem_u32(&tmem_base)) : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
   }
   fence_before();
   __syncthreads();
   fence_after();
   const unsigned tmem = tmem_base;
   volatile int *fail = &s_fail;
   auto wait = [&](unsigned long long *bar, unsigned ph) {
      if (*fail) { return; }
      if (!mbar_wait(bar, ph, 1LL << 20)) { *fail = 1; }
   };
   auto arrive = [&](unsigned long long *bar) {
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
   };
   const int ntiles = (ne + S::EL - 1) / S::EL;

   if (warp == 16)
   {
      // ----------------------------------------------------- MMA issuer
      constexpr uint32_t ID_F = instr_desc(128, S::NC), ID_B = instr_desc(128, S::KF, true);
      constexpr unsigned LBO_A = S::M / 8 * 128, LBO_BF = S::NC / 8 * 128;
      const uint64_t x_lo = smem_desc(sbase + S::OFF_XL, LBO_A, 128);
      const uint64_t tf_hi = smem_desc(sbase + S::OFF_T, LBO_BF, 128);
      const uint64_t tf_lo = smem_desc(sbase + S::OFF_T + S::BF_LIMB, LBO_BF, 128);
      const uint64_t tb_hi = smem_desc(sbase + S::OFF_T, 128, LBO_BF);
      const uint64_t tb_lo = smem_desc(sbase + S::OFF_T + S::BF_LIMB, 128, LBO_BF);
      auto ring = [](int c) { return (uint64_t)((c % S::NT) * 2 * S::BF_LIMB >> 4); };
      unsigned ph_t[S::NT] = {}, ph_af = 0, ph_ab = 0, ph_dfree[2] = {0, 0};
      int it = 0;
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it)
      {
         wait(MB_AF, ph_af); ph_af ^= 1;
         if (lane == 0) { TCB_TRACE(it, 1006); }
         for (int c = 0; c <= S::NCH; ++c)
         {
            if (c < S::NCH)
            {
               wait(MB_T + c % S::NT, ph_t[c % S::NT]); ph_t[c % S::NT] ^= 1;
               if (c >= 2) { wait(MB_DFREE + (c & 1), ph_dfree[c & 1]); ph_dfree[c & 1] ^= 1; }
               fence_after();
               if (lane == 0) { TCB_TRACE(it, 16 * c + 0); }
               // forward: Gq = X K^T over the KF dofs; a K step of 16 is 8 TMEM
               // columns of the hi limb, two core columns (2 LBO_A bytes) of
               // the lo limb and of the table chunk (2 LBO_BF bytes)
               const unsigned d = tmem + ((c & 1) ? S::TF1 : S::TF0);
               const uint64_t bh = tf_hi + ring(c), bl = tf_lo + ring(c);
               __syncwarp();
               if (elect_one())
               {
                  if (!*fail)
                  {
#pragma unroll 2
                     for (int st = 0; st < S::KF / 16; ++st)
                     {
                        const unsigned ah = tmem + S::TXH + 8 * st;
                        const uint64_t oa = (uint64_t)(st * 2 * LBO_A >> 4), ob = (uint64_t)(st * 2 * LBO_BF >> 4);
                        mma_f16_ta(d, ah, bh + ob, ID_F, st > 0);
                        mma_f16_ta(d, ah, bl + ob, ID_F, true);
                        mma_f16(d, x_lo + oa, bh + ob, ID_F, true);
                     }
                  }
                  mma_commit(MB_FWD + (c & 1));
               }
               __syncwarp();
            }
            if (c >= 1)
            {
               const int cb = c - 1;   // the chunk whose backward GEMM is issued
               if (c == S::NCH)
               {
                  // the epilogue's last two releases of the forward buffers
                  wait(MB_DFREE + (S::NCH & 1), ph_dfree[S::NCH & 1]); ph_dfree[S::NCH & 1] ^= 1;
                  wait(MB_DFREE + ((S::NCH - 1) & 1), ph_dfree[(S::NCH - 1) & 1]);
                  ph_dfree[(S::NCH - 1) & 1] ^= 1;
               }
               wait(MB_AB, ph_ab); ph_ab ^= 1;
               fence_after();
               if (lane == 0) { TCB_TRACE(it, 16 * cb + 1); }
               // backward: Y += O K over chunk cb (A: its O limbs in TMEM; B:
               // its table chunk, still in the ring, read MN-major)
               const uint64_t bh = tb_hi + ring(cb), bl = tb_lo + ring(cb);
               __syncwarp();
               if (elect_one())
               {
                  if (!*fail)
                  {
#pragma unroll
                     for (int st = 0; st < S::NC / 16; ++st)
                     {
                        const unsigned ah = tmem + S::TOH + 8 * st, al = tmem + S::TOL + 8 * st;
                        const uint64_t ob = (uint64_t)(st * 2 * 128 >> 4);
                        mma_f16_ta(tmem + S::TB, ah, bh + ob, ID_B, cb > 0 || st > 0);
                        mma_f16_ta(tmem + S::TB, ah, bl + ob, ID_B, true);
                        mma_f16_ta(tmem + S::TB, al, bh + ob, ID_B, true);
                     }
                  }
                  // the epilogue's O columns and the chunk's ring buffer (copy producer)
                  mma_commit(MB_BWD);
                  mma_commit(MB_TFREE + cb % S::NT);
               }
               __syncwarp();
            }
         }
      }
      // every MMA this warp issued has completed before TMEM is released
      __syncwarp();
      if (elect_one()) { mma_commit(MB_DRAIN); }
      __syncwarp();
      if (!mbar_wait(MB_DRAIN, 0, 1LL << 20)) { *fail = 1; }
   }
   else if (warp == 17)
   {
      // ---------------------------------------------------- copy producer
      if (lane == 0)
      {
         unsigned ph_tfree[S::NT] = {}, ph_qfree[2] = {0, 0};
         bool held_t[S::NT] = {}, held_q[2] = {false, false};
         int n_cp[S::NT + 2] = {};   // copies issued per barrier (ring 0-1, qdata 0-1)
         auto copy = [&](int slot, unsigned long long *bar, void *dst, const void *src, unsigned bytes) {
            if (*fail) { return; }
            mbar_expect(bar, bytes);
            bulk_g2s(dst, src, bytes, bar);
            ++n_cp[slot];
         };
         constexpr int QPF = 4;   // qdata chunks brought into L2 ahead of their copy
         auto prefetch_qd = [&](int tile, int c) {
            int t = tile, cc = c;
            if (cc >= S::NCH) { cc -= S::NCH; t += gridDim.x; }
            if (t < ntiles) { bulk_prefetch_l2(qT + ((size_t)t * S::NCH + cc) * S::QT_CHUNK, S::QD_BYTES); }
         };
         for (int k = 0; k < QPF; ++k) { prefetch_qd(blockIdx.x, k); }
         for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
         {
            // the next tile's gather map into L2 (its rows are contiguous;
            // a full tile's EL D^3 ints are a whole number of 16-byte units,
            // so the range starts 16-byte aligned when the map does)
            const long long en0 = (long long)(tile + gridDim.x) * S::EL;
            if (en0 + S::EL <= ne && (uintptr_t)gmap % 16 == 0)
            {
               bulk_prefetch_l2(gmap + en0 * S::D3, S::EL * S::D3 * 4);
            }
            for (int c = 0; c < S::NCH; ++c)
            {
               // qdata chunk c into buffer c % 2 once the epilogue has taken
               // the chunk held there; table chunk c into ring buffer c % NT
               // once the backward GEMM of the chunk held there has completed
               const int b = c & 1, k = c % S::NT;
               if (held_q[b]) { wait(MB_QFREE + b, ph_qfree[b]); ph_qfree[b] ^= 1; }
               held_q[b] = true;
               copy(S::NT + b, MB_QD + b, smem + S::OFF_QD + b * S::QD_BYTES,
                    qT + ((size_t)tile * S::NCH + c) * S::QT_CHUNK, S::QD_BYTES);
               prefetch_qd(tile, c + QPF);
               if (held_t[k]) { wait(MB_TFREE + k, ph_tfree[k]); ph_tfree[k] ^= 1; }
               held_t[k] = true;
               copy(k, MB_T + k, smem + S::off_t(c), tab_f + (size_t)c * 2 * S::BF_LIMB, 2 * S::BF_LIMB);
            }
         }
         // no bulk copy is still writing shared memory when the CTA exits
         for (int s = 0; s < S::NT + 2; ++s)
         {
            unsigned long long *bar = s < S::NT ? MB_T + s : MB_QD + (s - S::NT);
            if (n_cp[s] > 0 && !mbar_wait(bar, (unsigned)(n_cp[s] - 1) & 1u, 1LL << 20)) { *fail = 1; }
         }
      }
   }
   else
   {
      // ------------------------------------------------------- epilogue warps
      const unsigned lane_off = (unsigned)(32 * (warp & 3)) << 16;
      unsigned ph_qd[2] = {0, 0}, ph_fwd[2] = {0, 0}, ph_bwd = 0;
      const int el = r / R, rhs = r % R;
      // this thread's 16-byte core-matrix row in a K-major shared operand of
      // 128 rows: k group kg of row r
      auto core_row = [&](int kg) { return (kg * (S::M / 8) + (r >> 3)) * 128 + (r & 7) * 16; };
      const unsigned traw = tmem + lane_off + S::TB + part * S::KH;   // raw x staging (a tile's start)
      int it = 0;
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it)
      {
         const long long e0 = (long long)tile * S::EL;
         const long long e = e0 + el;
         const bool act = e < ne;
         if (tid == 0) { TCB_TRACE(it, 1000); }
         // ---- gather (ElementRestriction::Mult for R interleaved vectors):
         // batches of GW dofs, the next batch's map entries in flight while
         // this batch's values load; raw values into the result columns
         constexpr int GW = 16;
         constexpr int NB = (S::KH + GW - 1) / GW;
         const int *grow = gmap + e * S::D3 + part * S::KH;
         auto map_batch = [&](int g, int *gg) {
#pragma unroll
            for (int j = 0; j < GW; ++j)
            {
               const int k = GW * g + j, i = part * S::KH + k;
               gg[j] = (act && k < S::KH && i < S::D3) ? __ldg(grow + k) : GBPA_GATHER_SKIP;
            }
         };
         float m = 0.f;
         int gcur[GW], gnext[GW];
         map_batch(0, gcur);
#pragma unroll 1
         for (int g = 0; g < NB; ++g)
         {
            if (g + 1 < NB) { map_batch(g + 1, gnext); }
            float v[GW];
#pragma unroll
            for (int j = 0; j < GW; ++j)
            {
               const int gj = gcur[j];
               const int dof = gj == GBPA_GATHER_SKIP ? 0 : (gj >= 0 ? gj : -1 - gj);
               v[j] = __ldg(x + (long long)dof * R + rhs);
            }
            unsigned u[GW];
#pragma unroll
            for (int j = 0; j < GW; ++j)
            {
               const int gj = gcur[j];
               float w = gj >= 0 ? v[j] : -v[j];
               if (gj == GBPA_GATHER_SKIP) { w = 0.f; }
               else if (mask && __ldg(mask + (gj >= 0 ? gj : -1 - gj))) { w = 0.f; }
               m = fmaxf(m, fabsf(w));
               u[j] = __float_as_uint(w);
            }
            __syncwarp();   // converged for the warp-collective TMEM stores
#pragma unroll
            for (int q = 0; q < GW / 8; ++q)
            {
               if (GW * g + 8 * q < S::KH) { tmem_st8(traw + GW * g + 8 * q, u + 8 * q); }
            }
#pragma unroll
            for (int j = 0; j < GW; ++j) { gcur[j] = gnext[j]; }
         }
         if (tid == 0) { TCB_TRACE(it, 1001); }
         s_max[part][r] = m;
         asm volatile("bar.sync 1, %0;" ::"n"(S::EPI) : "memory");
         float sx = 1.f;
         {
            const float mm = fmaxf(fmaxf(s_max[0][r], s_max[1][r]), fmaxf(s_max[2][r], s_max[3][r]));
            if (mm > 0.f && mm <= 3.0e38f)
            {
               int ex;
               frexpf(mm, &ex);              // mm < 2^ex
               sx = ldexpf(1.f, 14 - ex);    // mm * sx in [2^13, 2^14)
            }
         }
         const float so = act ? __ldg(qscale + e) : 1.f;
         // the raw values become scaled limbs: hi into TMEM, lo into shared memory
         tmem_wait_st();
#pragma unroll 2
         for (int g8 = 0; g8 < S::KH / 8; ++g8)
         {
            float v[8];
            tmem_ld8(traw + 8 * g8, v);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; ++j) { v[j] *= sx; }
            uint4 hi, lo;
            split8(v, hi, lo);
            const unsigned h4[4] = {hi.x, hi.y, hi.z, hi.w};
            tmem_st4(tmem + lane_off + S::TXH + part * (S::KH / 2) + 4 * g8, h4);
            *reinterpret_cast<uint4 *>(smem + S::OFF_XL + core_row(part * (S::KH / 8) + g8)) = lo;
         }
         tmem_wait_st();
         fence_before();
         fence_async_smem();   // the forward GEMMs read the lo limb through the async proxy
         if (tid == 0) { TCB_TRACE(it, 1002); }
         arrive(MB_AF);

         // ---- chunks. Meanwhile the next tile's x is brought into L2: in
         // chunk c this thread loads its map entries of group c (8 dofs)
         // and prefetches the x lines of group c - 1, whose entries arrived
         // during the previous chunk.
         const long long enx = e + (long long)gridDim.x * S::EL;   // this row's element in the next tile
         const bool pf = tile + (int)gridDim.x < ntiles && enx < ne;
         const int *gnrow = gmap + enx * S::D3 + part * S::KH;
         int pm[8];
         auto chunk = [&](int c, int b) {
            // b = c & 1 (compile-time in each unrolled copy)
            wait(MB_QD + b, ph_qd[b]); ph_qd[b] ^= 1;
            if (tid == 0) { TCB_TRACE(it, 16 * c + 5); }
            const float *sq = reinterpret_cast<const float *>(smem + S::OFF_QD + b * S::QD_BYTES) +
                              part * S::NQ * S::EL + el;
            float qc[S::NQ];
#pragma unroll
            for (int k = 0; k < S::NQ; ++k) { qc[k] = sq[k * S::EL]; }
            fence_async_smem();
            arrive(MB_QFREE + b);
            if (pf && c <= S::KH / 8)
            {
               if (c >= 1)
               {
#pragma unroll
                  for (int j = 0; j < 8; ++j)
                  {
                     const int gj = pm[j];
                     if (gj != GBPA_GATHER_SKIP) { prefetch_l2(x + (long long)(gj >= 0 ? gj : -1 - gj) * R + rhs); }
                  }
               }
               if (c < S::KH / 8)
               {
#pragma unroll
                  for (int j = 0; j < 8; ++j)
                  {
                     const int k = 8 * c + j;
                     pm[j] = part * S::KH + k < S::D3 ? __ldg(gnrow + k) : GBPA_GATHER_SKIP;
                  }
               }
            }
            wait(MB_FWD + b, ph_fwd[b]); ph_fwd[b] ^= 1;
            if (tid == 0) { TCB_TRACE(it, 16 * c + 6); }
            __syncwarp();   // the warp-collective TMEM loads need the converged warp
            fence_after();
            float gq[S::NV];
            const unsigned tcol = tmem + lane_off + (b ? S::TF1 : S::TF0) + part * S::NV;
            tmem_ld8(tcol, gq);
            tmem_ld4(tcol + 8, gq + 8);
            tmem_wait_ld();
            fence_before();
            arrive(MB_DFREE + b);
            float o[S::NV];
#pragma unroll
            for (int p = 0; p < S::NP; ++p)
            {
               // qdata entries 11, 12, 13, 22, 23, 33 of point p
               const float O11 = qc[6 * p], O12 = qc[6 * p + 1], O13 = qc[6 * p + 2];
               const float O22 = qc[6 * p + 3], O23 = qc[6 * p + 4], O33 = qc[6 * p + 5];
               const float gx = gq[3 * p], gy = gq[3 * p + 1], gz = gq[3 * p + 2];
               o[3 * p] = (O11 * gx + O12 * gy + O13 * gz) * so;
               o[3 * p + 1] = (O12 * gx + O22 * gy + O23 * gz) * so;
               o[3 * p + 2] = (O13 * gx + O23 * gy + O33 * gz) * so;
            }
            if (tid == 0) { TCB_TRACE(it, 16 * c + 7); }
            // the O columns were last read by the backward GEMM of chunk c - 1
            if (c >= 1) { wait(MB_BWD, ph_bwd); ph_bwd ^= 1; }
            if (tid == 0) { TCB_TRACE(it, 16 * c + 8); }
            __syncwarp();
            {
               // 12 values: 6 columns per limb
               uint4 hi, lo;
               split8(o, hi, lo);
               const unsigned col = lane_off + part * (S::NV / 2);
               const unsigned h4[4] = {hi.x, hi.y, hi.z, hi.w}, l4[4] = {lo.x, lo.y, lo.z, lo.w};
               tmem_st4(tmem + S::TOH + col, h4);
               tmem_st4(tmem + S::TOL + col, l4);
               unsigned h2[2], l2[2];
               split4(o + 8, h2, l2);
               tmem_st2(tmem + S::TOH + col + 4, h2);
               tmem_st2(tmem + S::TOL + col + 4, l2);
            }
            tmem_wait_st();
            fence_before();
            if (tid == 0) { TCB_TRACE(it, 16 * c + 9); }
            arrive(MB_AB);
         };
#pragma unroll 1
         for (int c = 0; c < S::NCH; c += 2)
         {
            chunk(c, 0);
            chunk(c + 1, 1);
         }
         // ---- result: the tile's last backward GEMM has completed; undo
         // the scales and store
         wait(MB_BWD, ph_bwd); ph_bwd ^= 1;
         if (tid == 0) { TCB_TRACE(it, 1003); }
         __syncwarp();
         fence_after();
         const bool failed = *fail != 0;
         const float inv = failed ? NAN : 1.f / (sx * so);
         float *yrow = y + e * (long long)(S::D3 * R) + rhs;
#pragma unroll 2
         for (int j = 0; j < S::KH; j += 8)
         {
            float v[8];
            tmem_ld8(tmem + lane_off + S::TB + part * S::KH + j, v);
            tmem_wait_ld();
#pragma unroll
            for (int k = 0; k < 8; ++k)
            {
               const int i = part * S::KH + j + k;
               if (act && i < S::D3) { yrow[i * R] = v[k] * inv; }
            }
         }
         // the result columns are read before the next tile's gather writes them
         fence_before();
         if (tid == 0) { TCB_TRACE(it, 1005); }
      }
   }
   __syncthreads();
   if (tid == 0 && s_fail) { atomicOr(flags, GBPA_FLAG_TIMEOUT); }
   fence_before();
   __syncthreads();
   if (warp == 0)
   {
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
   }
}

// ------------------------------------------------------------- host side
// (D, Q, PC, R) with a block tensor-core kernel
#define GBPA_TC_BLOCK_LIST(X) X(5, 6, 16, 8) X(6, 7, 16, 8)

bool block_supported(int D, int Q, int nrhs)
{
#define GBPA_CASE(d, q, pc, rr) if (D == d && Q == q && nrhs == rr) { return true; }
   GBPA_TC_BLOCK_LIST(GBPA_CASE)
#undef GBPA_CASE
   return false;
}

int build_block_tables(int D, int Q, const double *B, const double *G, Tables *t)
{
#define GBPA_CASE(d, q, pc, rr)                                                                  \
   if (D == d && Q == q)                                                                        \
   {                                                                                            \
      std::vector<unsigned char> tf;                                                            \
      double Rb = 0.0;                                                                          \
      build_kron_tables(d, q, pc, B, G, tf, Rb);                                                \
      t->D = D; t->Q = Q; t->R = Rb;                                                            \
      int rc = check_cuda(cudaMalloc(&t->fwd, tf.size()), "cudaMalloc(tc block tables)");       \
      if (!rc)                                                                                  \
      {                                                                                         \
         rc = check_cuda(cudaMemcpy(t->fwd, tf.data(), tf.size(), cudaMemcpyHostToDevice),      \
                         "copy tc block tables");                                               \
      }                                                                                         \
      if (rc) { free_tables(t); }                                                               \
      return rc;                                                                                \
   }
   GBPA_TC_BLOCK_LIST(GBPA_CASE)
#undef GBPA_CASE
   return GBPA_ERR_UNSUPPORTED;
}

// qdata (Q^3, 6, NE) -> the block kernel's layout: tile t (EL elements),
// chunk c, part h of the row, value k = 6 p + s (point q = c PC + h NP + p, symmetric
// entry s), element el of the tile; padded points and elements are zero.
template <int D, int Q, int PC, int R>
__global__ void transpose_qdata_block_kernel(int ne, const float *__restrict__ qd, float *__restrict__ qT, int64_t n)
{
   using S = BShape<D, Q, PC, R>;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
   {
      const int el = (int)(i % S::EL);
      int64_t t = i / S::EL;
      const int k = (int)(t % S::NQ); t /= S::NQ;
      const int h = (int)(t % S::PARTS); t /= S::PARTS;
      const int c = (int)(t % S::NCH);
      const int64_t tile = t / S::NCH;
      const int p = k / 6, sidx = k % 6;
      const int q = c * PC + h * S::NP + p;
      const int64_t e = tile * S::EL + el;
      qT[i] = (e < ne && q < S::Q3) ? qd[(e * 6 + sidx) * S::Q3 + q] : 0.f;
   }
}

int64_t block_qdata_size(int D, int Q, int nrhs, int ne)
{
#define GBPA_CASE(d, q, pc, rr)                                                              \
   if (D == d && Q == q && nrhs == rr)                                                      \
   {                                                                                        \
      using S = BShape<d, q, pc, rr>;                                                       \
      return (int64_t)((ne + S::EL - 1) / S::EL) * S::NCH * S::QT_CHUNK;                    \
   }
   GBPA_TC_BLOCK_LIST(GBPA_CASE)
#undef GBPA_CASE
   return 0;
}

int launch_block_transpose_qdata(gbpa_ctx *ctx, int ne, int D, int Q, int nrhs, const float *qd, float *qT)
{
   if (ne <= 0) { return GBPA_SUCCESS; }
#define GBPA_CASE(d, q, pc, rr)                                                                       \
   if (D == d && Q == q && nrhs == rr)                                                               \
   {                                                                                                 \
      const int64_t n = block_qdata_size(D, Q, nrhs, ne);                                            \
      transpose_qdata_block_kernel<d, q, pc, rr><<<grid_for(n, 256, 16 * ctx->num_sms), 256, 0,      \
                                                   ctx->stream>>>(ne, qd, qT, n);                    \
      return last_launch(ctx, "tc_block_transpose_qdata");                                           \
   }
   GBPA_TC_BLOCK_LIST(GBPA_CASE)
#undef GBPA_CASE
   return GBPA_ERR_UNSUPPORTED;
}

template <int D, int Q, int PC, int R>
static int launch_block_t(gbpa_ctx *ctx, int ne, const Tables &t, const float *qT, const float *qscale,
                          const float *x, const int *gmap, const unsigned char *mask, float *y, const int *skip)
{
   using S = BShape<D, Q, PC, R>;
   const void *k = (const void *)diffusion_tc_block_kernel<D, Q, PC, R>;
   const int ntiles = (ne + S::EL - 1) / S::EL;
   const int grid = std::min(ntiles, ctx->num_sms > 0 ? ctx->num_sms : 148);
   const unsigned char *tf = t.fwd;
   int *flags = ctx->d_flags;
   void *args[] = {&ne, (void *)&tf, (void *)&qT, (void *)&qscale, (void *)&x, (void *)&gmap,
                   (void *)&mask, &y, (void *)&skip, &flags};
   return launch_generic(ctx, k, dim3(grid), dim3(576), args, S::SMEM, "diffusion_tc_block");
}

int launch_diffusion_block_f32(gbpa_ctx *ctx, int ne, int D, int Q, int nrhs, const Tables &t, const float *qT,
                               const float *qscale, const float *x, const int *gmap, const unsigned char *mask,
                               float *y, const int *skip)
{
   if (ne == 0) { return GBPA_SUCCESS; }
   if (t.D != D || t.Q != Q || !t.fwd || !gmap) { return GBPA_ERR_UNSUPPORTED; }
#define GBPA_CASE(d, q, pc, rr)                                                                          \
   if (D == d && Q == q && nrhs == rr)                                                                  \
   {                                                                                                    \
      return launch_block_t<d, q, pc, rr>(ctx, ne, t, qT, qscale, x, gmap, mask, y, skip);              \
   }
   GBPA_TC_BLOCK_LIST(GBPA_CASE)
#undef GBPA_CASE
   return GBPA_ERR_UNSUPPORTED;
}

} // namespace tc
} // namespace gbpa

#ifdef GBPA_TC_TRACE
extern "C" int gbpa_tcb_trace_read(unsigned long long *out, int n)
{
   return cudaMemcpyFromSymbol(out, gbpa::tc::g_tcb_trace, sizeof(unsigned long long) * (size_t)n) == cudaSuccess
             ? 0
             : -3;
}
#endif
