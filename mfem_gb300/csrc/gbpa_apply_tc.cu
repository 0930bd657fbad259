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
// chunk's O columns back to TMEM, and the backward GEMM accumulates the
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
// The A operands (the x tile, the chunk's O columns) are fp16 limbs in TMEM,
// two values per column, lane = element. The table chunks (shared memory,
// canonical no-swizzle layouts) are described in gbpa_tc_ptx.cuh.
#include "gbpa_apply_kernels.cuh"
#include "gbpa_dispatch.cuh"
#include "gbpa_tc.cuh"
#include "gbpa_tc_ptx.cuh"

namespace gbpa
{
namespace tc
{

// Timeline probes for kernel development: compiled in only with
// -DGBPA_TC_TRACE (SM clock of CTA 0's first tiles into a device table).
#ifdef GBPA_TC_TRACE
__device__ unsigned long long g_tc_trace[2048];
#define TC_TRACE(it, i)                                                           \
   do                                                                             \
   {                                                                              \
      if (blockIdx.x == 0 && (it) < 2) { g_tc_trace[(it) * 1024 + (i)] = clock64(); } \
   } while (0)
#else
#define TC_TRACE(it, i) do { } while (0)
#endif

template <int D, int Q, int PC>
struct Shape
{
   static constexpr int D3 = D * D * D;
   static constexpr int KF = (D3 + 15) / 16 * 16;   // dofs, padded to the MMA K step
   static constexpr int PARTS = 4;                  // epilogue threads per element row
   static constexpr int EPI = 128 * PARTS;          // epilogue threads (16 warps)
   static constexpr int KP = KF / PARTS;            // dofs per part of a row
   static constexpr int Q3 = Q * Q * Q;
   static constexpr int NC = 3 * PC;                // chunk columns (points x 3 components)
   static constexpr int NCH = (Q3 + PC - 1) / PC;   // chunks
   static constexpr int NP = PC / PARTS;            // points of a chunk per thread
   static constexpr int NV = 3 * NP;                // chunk columns per thread
   static constexpr int NQ = 6 * NP;                // qdata values per thread and chunk
   static constexpr int M = 128;                    // elements per tile
   static constexpr int BF_LIMB = NC * KF * 2;      // one limb of a table chunk
   static constexpr int MAP_BYTES = M * D3 * 4;     // the tile's gather map
   // shared memory: a ring of NT table-chunk buffers (chunk c in buffer
   // c % NT; the forward GEMM reads a chunk K-major, the backward GEMM reads
   // the same bytes as an MN-major operand), the chunk's qdata (bulk-copied
   // one chunk ahead) and the next tile's gather map. The result is staged
   // over the ring and the qdata buffer after the tile's last GEMM.
   static constexpr int NT = 3;
   static constexpr int QD_BYTES = PARTS * NQ * M * 4;  // one tile-chunk of transposed qdata
   static constexpr int OFF_T = 0;
   static constexpr int OFF_QD = OFF_T + NT * 2 * BF_LIMB;
   static constexpr int OFF_MAP = OFF_QD + QD_BYTES;
   static constexpr int SMEM = OFF_MAP + MAP_BYTES;
   static constexpr int OFF_STG = 0;
   // tensor memory (512 columns): two forward accumulators, the result, and
   // the GEMMs' A operands -- the x tile and the chunk's O columns, fp16 hi and
   // lo limbs, two values per column (lane = element)
   static constexpr int TF0 = 0, TF1 = 64, TB = 128;
   static constexpr int TXH = 256, TXL = TXH + KF / 2, TOH = 384, TOL = TOH + NC / 2;
   static __device__ __forceinline__ int off_t(int c) { return OFF_T + (c % NT) * 2 * BF_LIMB; }
   // output staging: row stride D3; an even stride is
   // XOR-swizzled by the row (bank-conflict-free either way)
   static constexpr int STG = D3;
   static_assert(D3 % 2 == 1 || D3 % 32 == 0, "staging swizzle");
   static __device__ __forceinline__ int stg(int row, int i)
   {
      return row * STG + (D3 % 2 ? i : (i ^ (row & 31)));
   }
   static constexpr int QT_CHUNK = PARTS * NQ * M;  // floats of one tile-chunk of transposed qdata
   static_assert(KF <= 128 && NC <= 64 && NC % 16 == 0 && NV == 12 && KP % 8 == 0, "TMEM and MMA shapes");
   static_assert(M * STG * 4 <= OFF_MAP, "output staging must fit over the ring and the qdata buffer");
   static_assert(KF / 2 <= 64 && NC / 2 <= 64, "A operands in TMEM");
   static_assert(SMEM <= 220 * 1024, "shared memory");
   static_assert(MAP_BYTES % 16 == 0, "bulk copy size");
   static_assert(NCH >= NT, "the table ring is filled at the tile start");
};

// Persistent kernel: one CTA per SM walks tiles of 128 elements. Warps 0-15
// (512 threads) gather, split, apply the qdata and write the result: thread t
// owns element row r = 32 (warp % 4) + lane (its TMEM lane) and part
// warp / 4 (a quarter) of that row's columns. Warp 16 issues the MMAs (one
// elected lane), one thread of warp 17 the bulk copies (gather map, table and
// qdata chunks),
// each waiting only for what it needs. The tensor pipe
// runs forward(c + 1) while the CUDA cores apply the qdata of chunk c, and
// backward(c) while they start chunk c + 1 (two forward accumulators in TMEM).
// Every wait is bounded: after a first expiry no wait blocks, no further MMA
// or bulk copy is started, the outputs are NaN and GBPA_FLAG_TIMEOUT is
// raised; before the CTA exits, the MMA warp and the copy producer wait
// (bounded) for the work they already started, so that no copy lands in
// released shared memory and no MMA uses released TMEM.
template <int D, int Q, int PC>
__global__ void __launch_bounds__(576, 1)
diffusion_tc_kernel(int ne, const unsigned char *__restrict__ tab_f,
                    const float *__restrict__ qT, const float *__restrict__ qscale, const float *__restrict__ x,
                    const int *__restrict__ gmap, int map_bulk, const unsigned char *__restrict__ mask,
                    float *__restrict__ y, int mode, const int *__restrict__ skip, int *flags)
{
   using S = Shape<D, Q, PC>;
   if (skip && *skip) { return; }   // uniform per launch: the solver has finished
   extern __shared__ __align__(1024) unsigned char smem[];
   // mbarriers: map, table ring 0-2, qd (bulk copies); af, ab, dfree0/1,
   // qfree, out (one arrival per epilogue thread); fwd0/1, bwd, tfree0-2 (the ring
   // buffer's backward GEMM is done), drain (MMA commits)
   constexpr int NMB = 18;
   __shared__ __align__(8) unsigned long long mb[NMB];
   __shared__ unsigned tmem_base;
   __shared__ float s_max[4][128];
   __shared__ int s_fail;
   unsigned long long *MB_MAP = mb, *MB_T = mb + 1, *MB_QD = mb + 4, *MB_AF = mb + 5;
   unsigned long long *MB_AB = mb + 6, *MB_DFREE = mb + 7, *MB_QFREE = mb + 9, *MB_FWD = mb + 10;
   unsigned long long *MB_BWD = mb + 12, *MB_OUT = mb + 13, *MB_TFREE = mb + 14, *MB_DRAIN = mb + 17;
   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int part = (warp >> 2) & 3;   // epilogue warps 0-15: the part of the row's columns
   const int r = 32 * (warp & 3) + lane;
   const unsigned sbase = smem_u32(smem);

   if (tid == 0)
   {
      const unsigned E = S::EPI;
      const unsigned counts[NMB] = {1, 1, 1, 1, 1, E, E, E, E, E, 1, 1, 1, E, 1, 1, 1, 1};
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
   const int ntiles = (ne + 127) / 128;

   if (warp == 16)
   {
      // ----------------------------------------------------- MMA issuer
      // the whole warp runs the loop (waits, descriptors: warp-uniform);
      // one elected lane issues each batch of MMAs and its commit
      {
         constexpr uint32_t ID_F = instr_desc(128, S::NC), ID_B = instr_desc(128, S::KF, true);
         constexpr unsigned LBO_BF = S::NC / 8 * 128;
         // descriptors of the first K step; a step advances the start
         // address field (bits 0-13, 16-byte units)
         // table ring buffer k: + k * 2 BF_LIMB bytes
         const uint64_t tf_hi = smem_desc(sbase + S::OFF_T, LBO_BF, 128);
         const uint64_t tf_lo = smem_desc(sbase + S::OFF_T + S::BF_LIMB, LBO_BF, 128);
         const uint64_t tb_hi = smem_desc(sbase + S::OFF_T, 128, LBO_BF);
         const uint64_t tb_lo = smem_desc(sbase + S::OFF_T + S::BF_LIMB, 128, LBO_BF);
         auto ring = [](int c) { return (uint64_t)((c % S::NT) * 2 * S::BF_LIMB >> 4); };
         unsigned ph_t[S::NT] = {}, ph_af = 0, ph_ab = 0, ph_dfree[2] = {0, 0};
         int it = 0;
         for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it)
         {
            if (lane == 0) TC_TRACE(it, 1000);
            wait(MB_AF, ph_af); ph_af ^= 1;
            if (lane == 0) TC_TRACE(it, 1001);
            for (int c = 0; c <= S::NCH; ++c)
            {
               if (c < S::NCH)
               {
                  wait(MB_T + c % S::NT, ph_t[c % S::NT]); ph_t[c % S::NT] ^= 1;
                  if (c >= 2) { wait(MB_DFREE + (c & 1), ph_dfree[c & 1]); ph_dfree[c & 1] ^= 1; }
                  fence_after();
                  if (lane == 0) TC_TRACE(it, 16 * c + 0);
                  // forward: Gq = X K^T over the KF dofs, three limb products
                  const unsigned d = tmem + ((c & 1) ? S::TF1 : S::TF0);
                  const uint64_t bh = tf_hi + ring(c), bl = tf_lo + ring(c);
                  __syncwarp();
                  if (elect_one())
                  {
                     // after a timed-out wait no further MMA is issued (its
                     // operands may not have arrived); the commits still arrive
                     if (!*fail)
                     {
#pragma unroll
                        for (int st = 0; st < S::KF / 16; ++st)
                        {
                           // A = the x tile in TMEM: 16 fp16 per K step = 8 columns
                           const unsigned ah = tmem + S::TXH + 8 * st, al = tmem + S::TXL + 8 * st;
                           const uint64_t ob = (uint64_t)(st * 2 * LBO_BF >> 4);
                           mma_f16_ta(d, ah, bh + ob, ID_F, st > 0);
                           mma_f16_ta(d, ah, bl + ob, ID_F, true);
                           mma_f16_ta(d, al, bh + ob, ID_F, true);
                        }
                     }
                     mma_commit(MB_FWD + (c & 1));
                  }
                  __syncwarp();
               }
               if (c >= 1)
               {
                  if (c == S::NCH)
                  {
                     // the epilogue's last two releases of the forward buffers
                     wait(MB_DFREE + (S::NCH & 1), ph_dfree[S::NCH & 1]); ph_dfree[S::NCH & 1] ^= 1;
                     wait(MB_DFREE + ((S::NCH - 1) & 1), ph_dfree[(S::NCH - 1) & 1]);
                     ph_dfree[(S::NCH - 1) & 1] ^= 1;
                  }
                  wait(MB_AB, ph_ab); ph_ab ^= 1;
                  fence_after();
                  if (lane == 0) TC_TRACE(it, 16 * (c - 1) + 1);
                  // backward: Y += O K over chunk c - 1's columns (its table
                  // chunk, still in the ring, read MN-major)
                  const uint64_t bh = tb_hi + ring(c - 1), bl = tb_lo + ring(c - 1);
                  __syncwarp();
                  if (elect_one())
                  {
                     if (!*fail)
                     {
#pragma unroll
                        for (int st = 0; st < S::NC / 16; ++st)
                        {
                           // A = the chunk's O columns in TMEM
                           const unsigned ah = tmem + S::TOH + 8 * st, al = tmem + S::TOL + 8 * st;
                           const uint64_t ob = (uint64_t)(st * 2 * 128 >> 4);
                           mma_f16_ta(tmem + S::TB, ah, bh + ob, ID_B, c > 1 || st > 0);
                           mma_f16_ta(tmem + S::TB, ah, bl + ob, ID_B, true);
                           mma_f16_ta(tmem + S::TB, al, bh + ob, ID_B, true);
                        }
                     }
                     // the epilogue's O buffer, and the chunk's ring buffer
                     // (its own barrier: the copy producer waits per buffer)
                     mma_commit(MB_BWD);
                     mma_commit(MB_TFREE + (c - 1) % S::NT);
                  }
                  __syncwarp();
               }
            }
         }
         // every MMA this warp issued has completed before TMEM is released
         // (a commit tracks all earlier MMAs of the issuing thread)
         __syncwarp();
         if (elect_one()) { mma_commit(MB_DRAIN); }
         __syncwarp();
         if (!mbar_wait(MB_DRAIN, 0, 1LL << 20)) { *fail = 1; }
      }
   }
   else if (warp == 17)
   {
      // ---------------------------------------------------- copy producer
      if (lane == 0)
      {
         unsigned ph_qfree = 0, ph_af = 0, ph_tfree[S::NT] = {};
         // copies issued per barrier (map, ring 0-2, qdata): each completes one
         // phase of its barrier, which nothing else arrives on
         int n_cp[2 + S::NT] = {};
         auto copy = [&](int slot, unsigned long long *bar, void *dst, const void *src, unsigned bytes) {
            if (*fail) { return; }   // after a timed-out wait nothing new is started
            mbar_expect(bar, bytes);
            bulk_g2s(dst, src, bytes, bar);
            ++n_cp[slot];
         };
         // table chunk c into ring buffer c % NT, once the backward GEMM of
         // the chunk held there before (if any) has completed
         bool held[S::NT] = {};
         auto load_t = [&](int c) {
            const int k = c % S::NT;
            if (held[k]) { wait(MB_TFREE + k, ph_tfree[k]); ph_tfree[k] ^= 1; }
            held[k] = true;
            copy(1 + k, MB_T + k, smem + S::off_t(c), tab_f + (size_t)c * 2 * S::BF_LIMB, 2 * S::BF_LIMB);
         };
         auto load_qd = [&](int tile, int c) {
            copy(1 + S::NT, MB_QD, smem + S::OFF_QD, qT + ((size_t)tile * S::NCH + c) * S::QT_CHUNK, S::QD_BYTES);
         };
         // qdata streams from HBM: the chunks QPF ahead of the one being
         // copied to shared memory are on their way into L2, so that copy is
         // an L2 hit (the next tile's chunks follow this tile's)
         constexpr int QPF = 3;
         auto prefetch_qd = [&](int tile, int c) {
            int t = tile, cc = c;
            if (cc >= S::NCH) { cc -= S::NCH; t += gridDim.x; }
            if (t < ntiles) { bulk_prefetch_l2(qT + ((size_t)t * S::NCH + cc) * S::QT_CHUNK, S::QD_BYTES); }
         };
         for (int k = 0; k < QPF; ++k) { prefetch_qd(blockIdx.x, k); }
         auto load_map = [&](int tile) {
            const long long e0 = (long long)tile * 128;
            if (tile < ntiles && map_bulk && e0 + 128 <= ne)
            {
               copy(0, MB_MAP, smem + S::OFF_MAP, gmap + e0 * S::D3, S::MAP_BYTES);
            }
         };
         unsigned ph_out = 0;
         load_map(blockIdx.x);
         int it = 0;
         for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it)
         {
            // the previous tile's GEMMs are done and its result has left the
            // staging over the ring and the qdata buffer (waited below)
            load_qd(tile, 0);
            for (int c = 0; c < S::NT && c < S::NCH; ++c) { load_t(c); }
            wait(MB_AF, ph_af); ph_af ^= 1;
            // this tile's map has been read: fetch the next tile's
            load_map(tile + gridDim.x);
            for (int c = 0; c < S::NCH; ++c)
            {
               // qdata chunk c + 1 once the epilogue has taken chunk c; table
               // chunk c + NT - 1 once bwd(c - 1) has freed its buffer
               wait(MB_QFREE, ph_qfree); ph_qfree ^= 1;
               if (c + 1 < S::NCH) { load_qd(tile, c + 1); }
               prefetch_qd(tile, c + QPF);
               if (c >= 1 && c + S::NT - 1 < S::NCH)
               {
                  load_t(c + S::NT - 1);
                  TC_TRACE(it, 16 * (c - 1) + 4);
               }
            }
            TC_TRACE(it, 1002);
            wait(MB_OUT, ph_out); ph_out ^= 1;   // the tile's result has been stored
         }
         // no bulk copy is still writing shared memory when the CTA exits: the
         // last phase each barrier was given has completed (earlier phases of a
         // barrier complete in order)
         for (int s = 0; s < 2 + S::NT; ++s)
         {
            unsigned long long *bar = s == 0 ? MB_MAP : (s <= S::NT ? MB_T + (s - 1) : MB_QD);
            if (n_cp[s] > 0 && !mbar_wait(bar, (unsigned)(n_cp[s] - 1) & 1u, 1LL << 20)) { *fail = 1; }
         }
      }
   }
   else
   {
      // ------------------------------------------------------- epilogue warps
      const unsigned lane_off = (unsigned)(32 * (warp & 3)) << 16;
      unsigned ph_map = 0, ph_qd = 0, ph_fwd[2] = {0, 0}, ph_bwd = 0;
      const int *smap = reinterpret_cast<const int *>(smem + S::OFF_MAP);
      float *stg = reinterpret_cast<float *>(smem + S::OFF_STG);
      int it = 0;
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it)
      {
         const long long e0 = (long long)tile * 128;
         const long long e = e0 + r;
         if (tid == 0) { TC_TRACE(it, 1010); }
         const bool act = e < ne;
         const bool bulk = map_bulk && e0 + 128 <= ne;
         // ---- gather this thread's part of the row of x (ElementRestriction::Mult)
         if (bulk) { wait(MB_MAP, ph_map); ph_map ^= 1; }
         // all map entries first, then all x loads (unconditional: a slot
         // without a dof reads x[0] and is zeroed by the select), so the
         // loads are in flight together
         int jj[S::KP];
         signed char sg[S::KP];
#pragma unroll
         for (int k = 0; k < S::KP; ++k)
         {
            const int i = part * S::KP + k;
            int g = GBPA_GATHER_SKIP;
            if (act && i < S::D3) { g = bulk ? smap[r * S::D3 + i] : __ldg(gmap + e * S::D3 + i); }
            const bool use = g != GBPA_GATHER_SKIP;
            jj[k] = use ? (g >= 0 ? g : -1 - g) : 0;
            sg[k] = use ? (g >= 0 ? 1 : -1) : 0;
         }
         if (mask)
         {
#pragma unroll
            for (int k = 0; k < S::KP; ++k)
            {
               if (__ldg(mask + jj[k])) { sg[k] = 0; }
            }
         }
         float xv[S::KP];
#pragma unroll
         for (int k = 0; k < S::KP; ++k) { xv[k] = __ldg(x + jj[k]); }
#pragma unroll
         for (int k = 0; k < S::KP; ++k) { xv[k] = sg[k] == 0 ? 0.f : (sg[k] > 0 ? xv[k] : -xv[k]); }
         float m = 0.f;
#pragma unroll
         for (int k = 0; k < S::KP; ++k) { m = fmaxf(m, fabsf(xv[k])); }
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
#pragma unroll
         // the x tile's fp16 limbs into TMEM (this thread's part of the row:
         // KP values, KP/2 columns per limb); the forward GEMMs read them as A
#pragma unroll
         for (int g8 = 0; g8 < S::KP / 8; ++g8)
         {
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) { v[j] = xv[8 * g8 + j] * sx; }
            uint4 hi, lo;
            split8(v, hi, lo);
            const unsigned col = lane_off + part * (S::KP / 2) + 4 * g8;
            const unsigned h4[4] = {hi.x, hi.y, hi.z, hi.w}, l4[4] = {lo.x, lo.y, lo.z, lo.w};
            tmem_st4(tmem + S::TXH + col, h4);
            tmem_st4(tmem + S::TXL + col, l4);
         }
         tmem_wait_st();
         fence_before();
         if (tid == 0) { TC_TRACE(it, 1011); }
         arrive(MB_AF);

         // ---- chunks: the producer bulk-copies chunk c's qdata (transposed
         // layout: this thread's 6 NP values at stride 128) into shared memory
         // one chunk ahead; it is taken into registers at the chunk's start
         const float *sq = reinterpret_cast<const float *>(smem + S::OFF_QD) + part * S::NQ * 128 + r;
#pragma unroll 1
         for (int c = 0; c < S::NCH; ++c)
         {
            wait(MB_QD, ph_qd); ph_qd ^= 1;
            if (tid == 0) { TC_TRACE(it, 16 * c + 5); }
            float qc[S::NQ];
#pragma unroll
            for (int k = 0; k < S::NQ; ++k) { qc[k] = sq[k * 128]; }
            fence_async_smem();
            arrive(MB_QFREE);
            wait(MB_FWD + (c & 1), ph_fwd[c & 1]); ph_fwd[c & 1] ^= 1;
            if (tid == 0) { TC_TRACE(it, 16 * c + 6); }
            __syncwarp();   // the warp-collective TMEM loads need the converged warp
            fence_after();
            float gq[S::NV];
            const unsigned tcol = tmem + lane_off + ((c & 1) ? S::TF1 : S::TF0) + part * S::NV;
            tmem_ld8(tcol, gq);
            tmem_ld4(tcol + 8, gq + 8);
            tmem_wait_ld();
            fence_before();
            arrive(MB_DFREE + (c & 1));
            float o[S::NV];
#pragma unroll
            for (int p = 0; p < S::NP; ++p)
            {
               // qdata entries 11, 12, 13, 22, 23, 33 of point p
               const float O11 = qc[6 * p], O12 = qc[6 * p + 1], O13 = qc[6 * p + 2];
               const float O22 = qc[6 * p + 3], O23 = qc[6 * p + 4], O33 = qc[6 * p + 5];
               const float gx = gq[3 * p], gy = gq[3 * p + 1], gz = gq[3 * p + 2];
               // the x scale stays in (undone at the output): |o so| < 2^14
               o[3 * p] = (O11 * gx + O12 * gy + O13 * gz) * so;
               o[3 * p + 1] = (O12 * gx + O22 * gy + O23 * gz) * so;
               o[3 * p + 2] = (O13 * gx + O23 * gy + O33 * gz) * so;
            }
            if (tid == 0) { TC_TRACE(it, 16 * c + 7); }
            if (c >= 1) { wait(MB_BWD, ph_bwd); ph_bwd ^= 1; }   // backward(c - 1) has read A_bwd
            __syncwarp();
            if (tid == 0) { TC_TRACE(it, 16 * c + 8); }
            // the chunk's O limbs into TMEM (NV = 12 values, 6 columns per limb)
            {
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
            arrive(MB_AB);
            if (tid == 0) { TC_TRACE(it, 16 * c + 9); }
         }
         // ---- result: D_bwd = (A_e x) sx so; undo the scales, stage, store
         wait(MB_BWD, ph_bwd); ph_bwd ^= 1;
         __syncwarp();
         if (tid == 0) { TC_TRACE(it, 1013); }
         fence_after();
         const float inv = 1.f / (sx * so);
#pragma unroll
         for (int j = 0; j < S::KP; j += 8)
         {
            float v[8];
            tmem_ld8(tmem + lane_off + S::TB + part * S::KP + j, v);
            tmem_wait_ld();
#pragma unroll
            for (int k = 0; k < 8; ++k)
            {
               const int i = part * S::KP + j + k;
               if (i < S::D3) { stg[S::stg(r, i)] = v[k] * inv; }
            }
         }
         fence_before();
         asm volatile("bar.sync 1, %0;" ::"n"(S::EPI) : "memory");
         const bool failed = *fail != 0;
         if (S::D3 % 2 == 1 && mode == 0 && !failed && e0 + 128 <= ne && ((uintptr_t)y % 16) == 0)
         {
            // an unswizzled full tile is the contiguous E-vector slice
            const float4 *src = reinterpret_cast<const float4 *>(stg);
            float4 *dst = reinterpret_cast<float4 *>(y + e0 * S::D3);
            for (int s = tid; s < 128 * S::D3 / 4; s += S::EPI) { dst[s] = src[s]; }
         }
         else
         for (int s = tid; s < 128 * S::D3; s += S::EPI)
         {
            const int el = s / S::D3, i = s - el * S::D3;
            const long long ee = e0 + el;
            if (ee >= ne) { continue; }
            const float v = failed ? NAN : stg[S::stg(el, i)];
            const long long slot = ee * S::D3 + i;
            store_result(y, slot, slot, v, mode, gmap, mask);
         }
         // the staging overlays the ring and the qdata buffer: release it to
         // the copy producer
         fence_async_smem();
         arrive(MB_OUT);
         if (tid == 0) { TC_TRACE(it, 1012); }
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
template <int D, int Q, int PC>
static void build_tables_t(const double *B, const double *G, std::vector<unsigned char> &tf, double &R)
{
   build_kron_tables(D, Q, PC, B, G, tf, R);
}

#define GBPA_TC_LIST(X) X(3, 4, 16) X(4, 5, 16) X(5, 6, 16)

bool supported(int D, int Q)
{
#define GBPA_CASE(d, q, pc) if (D == d && Q == q) { return true; }
   GBPA_TC_LIST(GBPA_CASE)
#undef GBPA_CASE
   return false;
}

int build_tables(int D, int Q, const double *B, const double *G, Tables *t)
{
   std::vector<unsigned char> tf;
   double R = 0.0;
   bool found = false;
#define GBPA_CASE(d, q, pc) \
   if (D == d && Q == q) { build_tables_t<d, q, pc>(B, G, tf, R); found = true; }
   GBPA_TC_LIST(GBPA_CASE)
#undef GBPA_CASE
   if (!found) { return GBPA_ERR_UNSUPPORTED; }
   t->D = D; t->Q = Q; t->R = R;
   int rc = check_cuda(cudaMalloc(&t->fwd, tf.size()), "cudaMalloc(tc tables)");
   if (!rc) { rc = check_cuda(cudaMemcpy(t->fwd, tf.data(), tf.size(), cudaMemcpyHostToDevice), "copy tc tables"); }
   if (rc) { free_tables(t); }
   return rc;
}

void free_tables(Tables *t)
{
   cudaFree(t->fwd);
   t->fwd = nullptr;
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

// qdata (Q^3, 6, NE) -> the kernel's tile layout: for tile t, chunk c, part h
// of the row, value k = 6 p + s (point q = c PC + h NP + p, symmetric entry s) the 128
// elements of the tile are consecutive; padded points and elements are zero.
template <int D, int Q, int PC>
__global__ void transpose_qdata_kernel(int ne, const float *__restrict__ qd, float *__restrict__ qT, int64_t n)
{
   using S = Shape<D, Q, PC>;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int r = (int)(i % 128);
      int64_t t = i / 128;
      const int k = (int)(t % S::NQ); t /= S::NQ;
      const int h = (int)(t % S::PARTS); t /= S::PARTS;
      const int c = (int)(t % S::NCH);
      const int64_t tile = t / S::NCH;
      const int p = k / 6, sidx = k % 6;
      const int q = c * PC + h * S::NP + p;
      const int64_t e = tile * 128 + r;
      qT[i] = (e < ne && q < S::Q3) ? qd[(e * 6 + sidx) * S::Q3 + q] : 0.f;
   }
}

template <int D, int Q, int PC>
static int64_t qt_size_t(int ne)
{
   using S = Shape<D, Q, PC>;
   return (int64_t)((ne + 127) / 128) * S::NCH * S::QT_CHUNK;
}

int64_t transposed_qdata_size(int D, int Q, int ne)
{
#define GBPA_CASE(d, q, pc) if (D == d && Q == q) { return qt_size_t<d, q, pc>(ne); }
   GBPA_TC_LIST(GBPA_CASE)
#undef GBPA_CASE
   return 0;
}

int launch_transpose_qdata(gbpa_ctx *ctx, int ne, int D, int Q, const float *qd, float *qT)
{
   if (ne <= 0) { return GBPA_SUCCESS; }
#define GBPA_CASE(d, q, pc)                                                                         \
   if (D == d && Q == q)                                                                            \
   {                                                                                                \
      const int64_t n = qt_size_t<d, q, pc>(ne);                                                    \
      transpose_qdata_kernel<d, q, pc><<<grid_for(n, 256, 16 * ctx->num_sms), 256, 0, ctx->stream>>>( \
         ne, qd, qT, n);                                                                            \
      return last_launch(ctx, "tc_transpose_qdata");                                                \
   }
   GBPA_TC_LIST(GBPA_CASE)
#undef GBPA_CASE
   return GBPA_ERR_UNSUPPORTED;
}

template <int D, int Q, int PC>
static int launch_t(gbpa_ctx *ctx, int ne, const Tables &t, const float *qT, const float *qscale, const float *x,
                    const int *gmap, const unsigned char *mask, float *y, int mode, const int *skip)
{
   using S = Shape<D, Q, PC>;
   const void *k = (const void *)diffusion_tc_kernel<D, Q, PC>;
   const int ntiles = (ne + 127) / 128;
   const int grid = std::min(ntiles, ctx->num_sms > 0 ? ctx->num_sms : 148);
   const unsigned char *tf = t.fwd;
   int *flags = ctx->d_flags;
   // the tile's map slice is bulk-copied when the map starts on a 16-byte
   // boundary (each full tile's slice then does too: 128 D^3 4 bytes)
   int map_bulk = ((uintptr_t)gmap % 16) == 0 ? 1 : 0;
   void *args[] = {&ne, (void *)&tf, (void *)&qT, (void *)&qscale, (void *)&x, (void *)&gmap,
                   &map_bulk, (void *)&mask, &y, &mode, (void *)&skip, &flags};
   return launch_generic(ctx, k, dim3(grid), dim3(576), args, S::SMEM, "diffusion_tc");
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

#ifdef GBPA_TC_TRACE
extern "C" int gbpa_tc_trace_read(unsigned long long *out, int n)
{
   return cudaMemcpyFromSymbol(out, gbpa::tc::g_tc_trace, sizeof(unsigned long long) * (size_t)n) == cudaSuccess ? 0
                                                                                                              : -3;
}
#endif
