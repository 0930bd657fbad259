// Batched PCG (batching form): many independent Dirichlet Poisson problems of
// uneven size and order solved together. Each problem follows CGSolver::Mult
// with OperatorJacobiSmoother (linalg/solvers.cpp:869-1050, 427-452) on its
// ConstrainedOperator-wrapped PA diffusion operator
// (linalg/operator.cpp:601-661, fem/bilinearform_ext.cpp:487-564); a converged
// problem drops out of the work while the others continue.
//
// Work decomposition (built on the host once per call):
//   element batches  (problem, first element, count): one block processes a
//                    batch with the 2D-slab layout (Q, Q, nbz) of that
//                    problem's order, nbz chosen per order (tuning table)
//   dof chunks       (problem, first dof, last dof): vector phases and the CSR
//                    scatter; each chunk writes one partial sum
// Per-problem dots sum their chunks' partials in chunk order, so results do
// not depend on the grid size or on scheduling.
//
// Two schedules run the same iteration:
//   graph       per iteration one grouped apply launch per order (that
//               order's compile-time kernel) and three vector-phase launches
//               over the active problems' chunks; the block that completes a
//               problem's partials finishes its scalars (last-block-done).
//               K iterations are captured in a CUDA graph; the host polls the
//               per-problem state between graph launches and rebuilds the
//               tables (and the graph) once the active elements have shrunk
//               enough, so converged problems stop costing blocks.
//   persistent  one cooperative launch for the whole solve with grid-wide
//               barriers between the phases and one runtime-size element
//               kernel. The grid barrier is a generation counter with a
//               bounded spin: a barrier that does not complete within the
//               spin budget raises GBPA_FLAG_TIMEOUT and every block leaves
//               the solve loop, so the kernel always terminates. The launch is
//               cooperative, so all blocks are co-resident and the barrier
//               completes in normal operation.
#include "gbpa_apply_kernels.cuh"
#include "gbpa_batched.cuh"
#include "gbpa_csr.cuh"
#include "gbpa_dispatch.cuh"
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

namespace gbpa
{
constexpr int BATCH_MAXD = 7;    // persistent schedule: p <= 6
constexpr int BATCH_MAXQ = 8;

int batched_apply_nbz_f64(int D, int Q);
int batched_apply_nbz_x2(int D, int Q);
int launch_batched_apply_f64(gbpa_ctx *ctx, int D, int Q, int nbz, const BBatch *batches, int nbatch,
                             const BProb *probs, const BScal *scal);
int launch_batched_apply_x2(gbpa_ctx *ctx, int D, int Q, int nbz, const BBatch *batches, int nbatch,
                            const BProb *probs, const BScal *scal);

int batched_apply_nbz(int precision, int D, int Q)
{
   return precision == GBPA_F64X2 ? batched_apply_nbz_x2(D, Q) : batched_apply_nbz_f64(D, Q);
}
int launch_batched_apply(gbpa_ctx *ctx, int precision, int D, int Q, int nbz, const BBatch *batches,
                         int nbatch, const BProb *probs, const BScal *scal)
{
   return precision == GBPA_F64X2 ? launch_batched_apply_x2(ctx, D, Q, nbz, batches, nbatch, probs, scal)
                                  : launch_batched_apply_f64(ctx, D, Q, nbz, batches, nbatch, probs, scal);
}

struct BParams
{
   const BProb *probs;
   BScal *scal;
   int nprob;
   const BBatch *batches;
   int nbatch;
   const BChunk *chunks;
   int nchunk;
   double *partials;
   double rel2, abs2;
   int max_it;
   unsigned int *bar_count;
   unsigned int *bar_gen;
   int *flags;
   int *n_active;
   int *abort;
   long long spin_limit;
};

// Sense-free generation barrier over all blocks, bounded spin.
__device__ bool grid_barrier(const BParams &P)
{
   __syncthreads();
   __shared__ int ok;
   if (threadIdx.x == 0)
   {
      ok = 1;
      volatile unsigned int *gen = P.bar_gen;
      const unsigned int g = *gen;
      __threadfence();
      if (atomicAdd(P.bar_count, 1u) == gridDim.x - 1)
      {
         *P.bar_count = 0;
         __threadfence();
         atomicAdd(P.bar_gen, 1u);
      }
      else
      {
         long long spins = 0;
         while (*gen == g)
         {
            if (*(volatile int *)P.abort) { ok = 0; break; }
            if (++spins > P.spin_limit)
            {
               atomicOr(P.flags, GBPA_FLAG_TIMEOUT);
               atomicExch(P.abort, 1);
               ok = 0;
               break;
            }
            __nanosleep(32);
         }
      }
      __threadfence();
   }
   __syncthreads();
   return ok != 0;
}

__device__ __forceinline__ double bwarp_sum(double v)
{
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) { v += __shfl_down_sync(0xffffffffu, v, o); }
   return v;
}
__device__ double bblock_sum(double v)
{
   __shared__ double ws[32];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   v = bwarp_sum(v);
   if (lane == 0) { ws[wid] = v; }
   __syncthreads();
   v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
   if (wid == 0) { v = bwarp_sum(v); }
   __syncthreads();
   return v;
}

// partials were written by other blocks: read through L2
__device__ double problem_sum(const BParams &P, const BProb &pr)
{
   double s = 0.0;
   for (int c = 0; c < pr.nchunk; ++c) { s += __ldcg(P.partials + pr.chunk0 + c); }
   return s;
}

// One batch's element apply: runtime-size code bounded by p <= 6 (a single
// variant keeps the persistent kernel free of register spills; per-order
// compile-time variants in one kernel spilled heavily).
template <typename AR>
__device__ __forceinline__ void batched_element(int D, int Q, long long e, bool active, bool part,
                                                int tx, int ty, const typename AR::V *sB,
                                                const typename AR::V *sG, typename AR::V *bufA,
                                                typename AR::V *bufB, const typename AR::Qd *qd,
                                                const double *d, const int *gmap,
                                                const unsigned char *mask, double *yE)
{
   diffusion_element<AR, 0, 0, true, BATCH_MAXD, BATCH_MAXQ, true>(
      e, active, part, D, Q, tx, ty, 1, sB, sG, bufA, bufB, qd, d, gmap, mask, yE, 0);
}

template <typename AR>
__global__ void __launch_bounds__(BATCH_THREADS)
batched_pcg_kernel(BParams P)
{
   using V = typename AR::V;
   extern __shared__ __align__(16) unsigned char smem_raw[];
   V *sm = reinterpret_cast<V *>(smem_raw);
   const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
   const int gthreads = gridDim.x * blockDim.x;
   volatile BScal *S = P.scal;

   // ---- init: r = b, x = 0, z = dinv r, d = z, partial (z, r)
   for (int c = blockIdx.x; c < P.nchunk; c += gridDim.x)
   {
      const BChunk ch = P.chunks[c];
      const BProb &pr = P.probs[ch.prob];
      double s = 0.0;
      for (int i = ch.i0 + threadIdx.x; i < ch.i1; i += blockDim.x)
      {
         const double ri = pr.b[i];
         pr.x[i] = 0.0;
         pr.r[i] = ri;
         const double zi = pr.dinv[i] * ri;
         pr.z[i] = zi;
         pr.d[i] = zi;
         s += zi * ri;
      }
      s = bblock_sum(s);
      if (threadIdx.x == 0) { P.partials[c] = s; }
   }
   if (gtid == 0) { *(volatile int *)P.n_active = 0; }
   if (!grid_barrier(P)) { return; }
   for (int k = gtid; k < P.nprob; k += gthreads)
   {
      volatile BScal &sc = S[k];
      const double nom = problem_sum(P, P.probs[k]);
      sc.nom = nom; sc.nom0 = nom; sc.betanom = nom;
      sc.iter = 1; sc.converged = 0; sc.final_iter = 0;
      int done = 0;
      if (!isfinite(nom)) { atomicOr(P.flags, GBPA_FLAG_NOT_FINITE); done = 1; }
      else if (nom < 0.0) { done = 1; }
      else
      {
         sc.r0 = fmax(nom * P.rel2, P.abs2);
         if (nom <= sc.r0) { sc.converged = 1; done = 1; }
      }
      sc.done = done;
      if (!done) { atomicAdd(P.n_active, 1); }
   }
   if (!grid_barrier(P)) { return; }

   for (int it = 0; ; ++it)
   {
      if (*(volatile int *)P.n_active == 0) { break; }
      // ---- A: yE = A_e d (gather of d, written by other blocks, via L2)
      for (int bi = blockIdx.x; bi < P.nbatch; bi += gridDim.x)
      {
         const BBatch bt = P.batches[bi];
         if (S[bt.prob].done) { continue; }      // uniform over the block
         const BProb &pr = P.probs[bt.prob];
         const int D = pr.D, Q = pr.Q;
         __syncthreads();                         // previous batch done with smem
         V *sB = sm, *sG = sm + Q * D;
         for (int i = threadIdx.x; i < Q * D; i += blockDim.x)
         {
            sB[(i % Q) * D + i / Q] = AR::in(pr.B[i]);
            sG[(i % Q) * D + i / Q] = AR::in(pr.G[i]);
         }
         const int t = threadIdx.x;
         const int tz = t / (Q * Q), tx = t % Q, ty = (t / Q) % Q;
         const bool part = tz < pr.nbz;
         const int per = diff_smem_per_elem(D, Q);
         V *bufA = sm + 2 * Q * D + (part ? tz : 0) * per;
         V *bufB = bufA + (per - 2 * D * D * Q);
         const typename AR::Qd *qd;
         // the split (hi, lo) copy for the double-float arithmetic, the FP64
         // qdata otherwise (select by type: both element types are 8 bytes)
         if constexpr (std::is_same<typename AR::Qd, float2>::value) { qd = pr.qd2; }
         else { qd = pr.qd; }
         batched_element<AR>(D, Q, (long long)bt.e0 + tz, part && tz < bt.count, part, tx, ty, sB, sG,
                             bufA, bufB, qd, pr.d, pr.gmap, nullptr, pr.yE);
      }
      if (!grid_barrier(P)) { return; }
      // ---- S: z = R^T yE (z[ess] = d[ess]); partial (d, z). yE comes from
      // other blocks (L2 loads); d and z of a chunk belong to this block.
      for (int c = blockIdx.x; c < P.nchunk; c += gridDim.x)
      {
         const BChunk ch = P.chunks[c];
         if (S[ch.prob].done) { continue; }
         const BProb &pr = P.probs[ch.prob];
         double s = 0.0;
         for (int i = ch.i0 + threadIdx.x; i < ch.i1; i += blockDim.x)
         {
            double v;
            if (pr.mask && pr.mask[i]) { v = pr.d[i]; }
            else { v = csr_row_sum<double, true>(pr.off, pr.ind, pr.yE, i); }
            pr.z[i] = v;
            s += pr.d[i] * v;
         }
         s = bblock_sum(s);
         if (threadIdx.x == 0) { P.partials[c] = s; }
      }
      if (!grid_barrier(P)) { return; }
      for (int k = gtid; k < P.nprob; k += gthreads)
      {
         volatile BScal &sc = S[k];
         if (sc.done) { continue; }
         const double den = problem_sum(P, P.probs[k]);
         sc.den = den;
         if (!isfinite(den)) { atomicOr(P.flags, GBPA_FLAG_NOT_FINITE); sc.final_iter = sc.iter; sc.done = 1; }
         else if (den == 0.0) { sc.final_iter = sc.iter; sc.done = 1; }
         else
         {
            if (it > 0) { sc.nom = sc.betanom; }
            sc.alpha = sc.nom / den;
         }
      }
      if (gtid == 0) { *(volatile int *)P.n_active = 0; }
      if (!grid_barrier(P)) { return; }
      // ---- U: x += alpha d; r -= alpha z; z = dinv r; partial (r, z)
      for (int c = blockIdx.x; c < P.nchunk; c += gridDim.x)
      {
         const BChunk ch = P.chunks[c];
         if (S[ch.prob].done) { continue; }
         const BProb &pr = P.probs[ch.prob];
         const double alpha = S[ch.prob].alpha;
         double s = 0.0;
         for (int i = ch.i0 + threadIdx.x; i < ch.i1; i += blockDim.x)
         {
            pr.x[i] += alpha * pr.d[i];
            const double ri = pr.r[i] - alpha * pr.z[i];
            pr.r[i] = ri;
            const double zi = pr.dinv[i] * ri;
            pr.z[i] = zi;
            s += ri * zi;
         }
         s = bblock_sum(s);
         if (threadIdx.x == 0) { P.partials[c] = s; }
      }
      if (!grid_barrier(P)) { return; }
      for (int k = gtid; k < P.nprob; k += gthreads)
      {
         volatile BScal &sc = S[k];
         if (sc.done) { continue; }
         const double bn = problem_sum(P, P.probs[k]);
         sc.betanom = bn;
         int done = 0;
         if (!isfinite(bn)) { atomicOr(P.flags, GBPA_FLAG_NOT_FINITE); sc.final_iter = sc.iter; done = 1; }
         else if (bn < 0.0) { sc.final_iter = sc.iter; done = 1; }
         else if (bn <= sc.r0) { sc.converged = 1; sc.final_iter = sc.iter; done = 1; }
         else
         {
            const int iter = sc.iter + 1;
            sc.iter = iter;
            if (iter > P.max_it) { sc.final_iter = P.max_it; done = 1; }
            else { sc.beta = bn / sc.nom; }
         }
         sc.done = done;
         if (!done) { atomicAdd(P.n_active, 1); }
      }
      if (!grid_barrier(P)) { return; }
      // ---- direction: d = z + beta d (chunk-owned vectors)
      for (int c = blockIdx.x; c < P.nchunk; c += gridDim.x)
      {
         const BChunk ch = P.chunks[c];
         if (S[ch.prob].done) { continue; }
         const BProb &pr = P.probs[ch.prob];
         const double beta = S[ch.prob].beta;
         for (int i = ch.i0 + threadIdx.x; i < ch.i1; i += blockDim.x)
         {
            pr.d[i] = pr.z[i] + beta * pr.d[i];
         }
      }
      if (!grid_barrier(P)) { return; }
   }
}

__global__ void batched_mask_kernel(int n, const int *ess, unsigned char *mask, int ndofs, int *flags)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
   {
      const int k = ess[i];
      if (k < 0 || k >= ndofs) { atomicOr(flags, GBPA_FLAG_INDEX); continue; }
      mask[k] = 1;
   }
}

// ------------------------------------------------------------ graph schedule
struct GParams
{
   const BProb *probs;
   BScal *scal;
   const BChunk *chunks;
   double *partials;
   unsigned int *cnt;   // per problem: chunks of the current phase published
   double rel2, abs2;
   int max_it;
   int *flags;
};

// Publishes a chunk's partial (thread 0 holds the block sum) and returns, in
// thread 0, whether this block completed its problem's set of partials. Then
// (thread 0 only) problem_total sums them in chunk order and re-arms the
// counter for the next phase.
__device__ __forceinline__ bool chunk_publish(const GParams &P, const BChunk &ch, int nchunk, double s)
{
   bool last = false;
   if (threadIdx.x == 0)
   {
      P.partials[ch.slot] = s;
      __threadfence();
      last = atomicAdd(P.cnt + ch.prob, 1u) == (unsigned)(nchunk - 1);
   }
   return last;
}
__device__ __forceinline__ double problem_total(const GParams &P, const BProb &pr, int prob)
{
   __threadfence();
   double s = 0.0;
   for (int c = 0; c < pr.nchunk; ++c) { s += __ldcg(P.partials + pr.chunk0 + c); }
   P.cnt[prob] = 0;
   return s;
}

// r = b, x = 0, z = dinv r, d = z; nom = (z, r), stopping threshold
__global__ void __launch_bounds__(BATCH_THREADS) bg_init_kernel(GParams P)
{
   const BChunk ch = P.chunks[blockIdx.x];
   const BProb &pr = P.probs[ch.prob];
   double s = 0.0;
   for (int i = ch.i0 + threadIdx.x; i < ch.i1; i += blockDim.x)
   {
      const double ri = pr.b[i];
      pr.x[i] = 0.0;
      pr.r[i] = ri;
      const double zi = pr.dinv[i] * ri;
      pr.z[i] = zi;
      pr.d[i] = zi;
      s += zi * ri;
   }
   s = bblock_sum(s);
   if (chunk_publish(P, ch, pr.nchunk, s))
   {
      BScal &sc = P.scal[ch.prob];
      const double nom = problem_total(P, pr, ch.prob);
      sc.nom = nom; sc.nom0 = nom; sc.betanom = nom;
      sc.iter = 1; sc.converged = 0; sc.final_iter = 0;
      int done = 0;
      if (!isfinite(nom)) { atomicOr(P.flags, GBPA_FLAG_NOT_FINITE); done = 1; }
      else if (nom < 0.0) { done = 1; }
      else
      {
         sc.r0 = fmax(nom * P.rel2, P.abs2);
         if (nom <= sc.r0) { sc.converged = 1; done = 1; }
      }
      sc.done = done;
   }
}

// z = R^T yE (z[ess] = d[ess]); den = (d, z); alpha = nom / den
__global__ void __launch_bounds__(BATCH_THREADS) bg_scatter_den_kernel(GParams P)
{
   const BChunk ch = P.chunks[blockIdx.x];
   if (P.scal[ch.prob].done) { return; }
   const BProb &pr = P.probs[ch.prob];
   double s = 0.0;
   for (int i = ch.i0 + threadIdx.x; i < ch.i1; i += blockDim.x)
   {
      double v;
      if (pr.mask && pr.mask[i]) { v = pr.d[i]; }
      else { v = csr_row_sum<double>(pr.off, pr.ind, pr.yE, i); }
      pr.z[i] = v;
      s += pr.d[i] * v;
   }
   s = bblock_sum(s);
   if (chunk_publish(P, ch, pr.nchunk, s))
   {
      BScal &sc = P.scal[ch.prob];
      const double den = problem_total(P, pr, ch.prob);
      sc.den = den;
      if (!isfinite(den)) { atomicOr(P.flags, GBPA_FLAG_NOT_FINITE); sc.final_iter = sc.iter; sc.done = 1; }
      else if (den == 0.0) { sc.final_iter = sc.iter; sc.done = 1; }
      else { sc.alpha = sc.nom / den; }
   }
}

// x += alpha d; r -= alpha z; z = dinv r; betanom = (r, z); convergence; beta
__global__ void __launch_bounds__(BATCH_THREADS) bg_update_kernel(GParams P)
{
   const BChunk ch = P.chunks[blockIdx.x];
   if (P.scal[ch.prob].done) { return; }
   const BProb &pr = P.probs[ch.prob];
   const double alpha = P.scal[ch.prob].alpha;
   double s = 0.0;
   for (int i = ch.i0 + threadIdx.x; i < ch.i1; i += blockDim.x)
   {
      pr.x[i] += alpha * pr.d[i];
      const double ri = pr.r[i] - alpha * pr.z[i];
      pr.r[i] = ri;
      const double zi = pr.dinv[i] * ri;
      pr.z[i] = zi;
      s += ri * zi;
   }
   s = bblock_sum(s);
   if (chunk_publish(P, ch, pr.nchunk, s))
   {
      BScal &sc = P.scal[ch.prob];
      const double bn = problem_total(P, pr, ch.prob);
      sc.betanom = bn;
      int done = 0;
      if (!isfinite(bn)) { atomicOr(P.flags, GBPA_FLAG_NOT_FINITE); sc.final_iter = sc.iter; done = 1; }
      else if (bn < 0.0) { sc.final_iter = sc.iter; done = 1; }
      else if (bn <= sc.r0) { sc.converged = 1; sc.final_iter = sc.iter; done = 1; }
      else
      {
         const int iter = sc.iter + 1;
         sc.iter = iter;
         if (iter > P.max_it) { sc.final_iter = P.max_it; done = 1; }
         else
         {
            sc.beta = bn / sc.nom;
            sc.nom = bn;
         }
      }
      sc.done = done;
   }
}

// d = z + beta d
__global__ void __launch_bounds__(BATCH_THREADS) bg_direction_kernel(GParams P)
{
   const BChunk ch = P.chunks[blockIdx.x];
   if (P.scal[ch.prob].done) { return; }
   const BProb &pr = P.probs[ch.prob];
   const double beta = P.scal[ch.prob].beta;
   for (int i = ch.i0 + threadIdx.x; i < ch.i1; i += blockDim.x)
   {
      pr.d[i] = pr.z[i] + beta * pr.d[i];
   }
}

} // namespace gbpa

namespace gbpa
{
namespace
{
struct Group { int D, Q, nbz; };

// The graph schedule's tables for the problems with active[k] set: element
// batches grouped by order (group g owns batches [gofs[g], gofs[g+1])) and
// the problems' dof chunks (each keeps its slot in the full chunk list).
void graph_tables(const std::vector<BProb> &hp, const std::vector<Group> &groups,
                  const std::vector<int> &grp_of, const std::vector<char> &active,
                  std::vector<BBatch> &batches, std::vector<int> &gofs, std::vector<BChunk> &chunks)
{
   batches.clear();
   chunks.clear();
   gofs.assign(groups.size() + 1, 0);
   for (size_t g = 0; g < groups.size(); ++g)
   {
      gofs[g] = (int)batches.size();
      const int nbz = groups[g].nbz;
      for (size_t k = 0; k < hp.size(); ++k)
      {
         if (!active[k] || grp_of[k] != (int)g) { continue; }
         for (int e0 = 0; e0 < hp[k].ne; e0 += nbz)
         {
            batches.push_back({(int)k, e0, std::min(nbz, hp[k].ne - e0)});
         }
      }
   }
   gofs[groups.size()] = (int)batches.size();
   for (size_t k = 0; k < hp.size(); ++k)
   {
      if (!active[k]) { continue; }
      for (int c = 0; c < hp[k].nchunk; ++c)
      {
         const int i0 = c * CHUNK;
         chunks.push_back({(int)k, i0, std::min(hp[k].ndofs, i0 + CHUNK), hp[k].chunk0 + c});
      }
   }
}

int check_every()
{
   const char *s = getenv("GBPA_PCG_CHECK_EVERY");
   const int k = s ? atoi(s) : 10;
   return k >= 1 && k <= 1000 ? k : 10;
}

// Runs the graph schedule from the uploaded tables to the end of the solve.
int run_graph_schedule(gbpa_ctx *ctx, int precision, const std::vector<BProb> &hp,
                       const std::vector<Group> &groups, const std::vector<int> &grp_of, GParams G,
                       BProb *d_probs, BBatch *d_batch, BChunk *d_chunk, int nchunk_all, int max_it,
                       std::vector<BScal> &hs, float *ms)
{
   const int nprob = (int)hp.size();
   int rc = GBPA_SUCCESS;
   if (!ctx->capture_stream)
   {
      rc = check_cuda(cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking),
                      "cudaStreamCreate(capture)");
      if (rc) { return rc; }
   }
   StreamTimer timer(ctx->stream);
   if (nchunk_all > 0)
   {
      bg_init_kernel<<<nchunk_all, BATCH_THREADS, 0, ctx->stream>>>(G);
      rc = last_launch(ctx, "batched_init");
   }
   const int K = check_every();
   cudaGraphExec_t exec = nullptr;
   int64_t table_elems = 0;
   int per_iter = 0;
   long long launched = 0;
   std::vector<BBatch> tb;
   std::vector<BChunk> tc;
   std::vector<int> gofs;
   std::vector<char> active(nprob, 0);
   while (!rc)
   {
      rc = check_cuda(cudaMemcpyAsync(hs.data(), G.scal, sizeof(BScal) * nprob, cudaMemcpyDeviceToHost,
                                      ctx->stream), "cudaMemcpyAsync(state)");
      if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize"); }
      if (rc) { break; }
      int64_t act_elems = 0;
      int nact = 0;
      for (int k = 0; k < nprob; ++k)
      {
         active[k] = hs[k].done ? 0 : 1;
         if (active[k]) { ++nact; act_elems += hp[k].ne; }
      }
      if (nact == 0) { break; }
      if (launched > (long long)max_it + K) { break; }   // safety net; the device caps iterations
      // (re)build the tables and the graph when the active elements have
      // fallen to 60% of those the current graph launches blocks for
      if (!exec || act_elems * 10 <= table_elems * 6)
      {
         graph_tables(hp, groups, grp_of, active, tb, gofs, tc);
         if (!tb.empty())
         {
            rc = check_cuda(cudaMemcpyAsync(d_batch, tb.data(), sizeof(BBatch) * tb.size(),
                                            cudaMemcpyHostToDevice, ctx->stream), "copy");
         }
         if (!rc && !tc.empty())
         {
            rc = check_cuda(cudaMemcpyAsync(d_chunk, tc.data(), sizeof(BChunk) * tc.size(),
                                            cudaMemcpyHostToDevice, ctx->stream), "copy");
         }
         if (rc) { break; }
         if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
         // capture on the private stream (the context's stream may be the
         // legacy default stream, which cannot be captured); captured
         // launches are not counted, executed ones are (below)
         const int64_t launches0 = ctx->launches;
         cudaGraph_t g = nullptr;
         cudaStream_t saved = ctx->stream;
         rc = check_cuda(cudaStreamBeginCapture(ctx->capture_stream, cudaStreamCaptureModeThreadLocal),
                         "cudaStreamBeginCapture");
         if (rc) { break; }
         ctx->stream = ctx->capture_stream;
         const unsigned nc = (unsigned)tc.size();
         per_iter = 3;
         for (size_t gi = 0; gi < groups.size(); ++gi) { per_iter += gofs[gi + 1] > gofs[gi] ? 1 : 0; }
         for (int it = 0; it < K && !rc; ++it)
         {
            for (size_t gi = 0; gi < groups.size() && !rc; ++gi)
            {
               const int cnt = gofs[gi + 1] - gofs[gi];
               if (cnt == 0) { continue; }
               rc = launch_batched_apply(ctx, precision, groups[gi].D, groups[gi].Q, groups[gi].nbz,
                                         d_batch + gofs[gi], cnt, d_probs, G.scal);
            }
            if (rc) { break; }
            bg_scatter_den_kernel<<<nc, BATCH_THREADS, 0, ctx->stream>>>(G);
            rc = last_launch(ctx, "batched_scatter_den");
            if (rc) { break; }
            bg_update_kernel<<<nc, BATCH_THREADS, 0, ctx->stream>>>(G);
            rc = last_launch(ctx, "batched_update");
            if (rc) { break; }
            bg_direction_kernel<<<nc, BATCH_THREADS, 0, ctx->stream>>>(G);
            rc = last_launch(ctx, "batched_direction");
         }
         ctx->stream = saved;
         ctx->launches = launches0;
         const int rc2 = check_cuda(cudaStreamEndCapture(ctx->capture_stream, &g), "cudaStreamEndCapture");
         if (rc || rc2)
         {
            if (g) { cudaGraphDestroy(g); }
            if (!rc) { rc = rc2; }
            break;
         }
         rc = check_cuda(cudaGraphInstantiate(&exec, g, 0), "cudaGraphInstantiate");
         cudaGraphDestroy(g);
         if (rc) { break; }
         table_elems = act_elems;
      }
      rc = check_cuda(cudaGraphLaunch(exec, ctx->stream), "cudaGraphLaunch");
      ctx->launches += (int64_t)K * per_iter;
      launched += K;
   }
   const float t = timer.stop(ctx->stream);
   if (exec) { cudaGraphExecDestroy(exec); }
   if (ms) { *ms = t; }
   return rc;
}
} // namespace

static int batched_solve(gbpa_ctx *ctx, int nprob, const gbpa_problem_desc *probs, int precision,
                         int schedule, double rel_tol, double abs_tol, int max_it, int *iterations,
                         int *converged, double *final_norms, double *seconds)
{
   if (precision != GBPA_F64 && precision != GBPA_F64X2) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (schedule != GBPA_BATCH_GRAPH && schedule != GBPA_BATCH_PERSISTENT) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (!ctx || nprob < 0 || (nprob > 0 && !probs) || max_it < 0 || rel_tol < 0 || abs_tol < 0)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (nprob == 0) { return GBPA_SUCCESS; }
   const bool graph = schedule == GBPA_BATCH_GRAPH;
   // ---- host tables
   std::vector<BProb> hp(nprob);
   std::vector<Group> groups;
   std::vector<int> grp_of(nprob, 0);
   std::vector<BBatch> batches;
   std::vector<BChunk> chunks;
   size_t ws_doubles = 0, mask_bytes = 0, gm_ints = 0;
   size_t smem_max = 0;
   for (int k = 0; k < nprob; ++k)
   {
      const gbpa_problem_desc &d = probs[k];
      if (d.ne < 0 || d.ndofs < 0 || d.n_ess < 0) { return GBPA_ERR_INVALID_ARGUMENT; }
      if (d.d1d < 1 || d.q1d < 1) { return GBPA_ERR_UNSUPPORTED; }
      if (d.n_ess > 0) { gm_ints += (size_t)d.ne * d.d1d * d.d1d * d.d1d; }
      if (!graph && (d.d1d > BATCH_MAXD || d.q1d > BATCH_MAXQ)) { return GBPA_ERR_UNSUPPORTED; }
      if (d.ne > 0 && (!d.B || !d.G || !d.qdata || !d.gather_map || !d.offsets || !d.indices)) { return GBPA_ERR_INVALID_ARGUMENT; }
      if (d.ndofs > 0 && (!d.dinv || !d.b || !d.x)) { return GBPA_ERR_INVALID_ARGUMENT; }
      if (d.n_ess > 0 && !d.ess) { return GBPA_ERR_INVALID_ARGUMENT; }
      const int Q = d.q1d, D = d.d1d;
      int nbz = 0;
      if (graph)
      {
         size_t g = 0;
         while (g < groups.size() && !(groups[g].D == D && groups[g].Q == Q)) { ++g; }
         if (g == groups.size())
         {
            const int nb = batched_apply_nbz(precision, D, Q);
            if (nb < 1) { return GBPA_ERR_UNSUPPORTED; }
            groups.push_back({D, Q, nb});
         }
         grp_of[k] = (int)g;
         nbz = groups[g].nbz;
      }
      else
      {
         nbz = std::max(1, std::min(elements_per_block(GBPA_DIFFUSION, GBPA_F64, D, Q), BATCH_THREADS / (Q * Q)));
         for (int e0 = 0; e0 < d.ne; e0 += nbz) { batches.push_back({k, e0, std::min(nbz, d.ne - e0)}); }
         const size_t sm = sizeof(double) * (2 * Q * D + (size_t)nbz * diff_smem_per_elem(D, Q));
         smem_max = std::max(smem_max, sm);
      }
      BProb &p = hp[k];
      p = BProb{};
      p.ne = d.ne; p.ndofs = d.ndofs; p.D = D; p.Q = Q; p.nbz = nbz;
      p.B = d.B; p.G = d.G; p.qd = d.qdata; p.dinv = d.dinv; p.b = d.b; p.x = d.x;
      p.gmap = d.gather_map; p.off = d.offsets; p.ind = d.indices;
      p.chunk0 = (int)chunks.size();
      for (int i0 = 0; i0 < d.ndofs; i0 += CHUNK)
      {
         chunks.push_back({k, i0, std::min(d.ndofs, i0 + CHUNK), (int)chunks.size()});
      }
      p.nchunk = (int)chunks.size() - p.chunk0;
      ws_doubles += 3 * (size_t)d.ndofs + (size_t)d.ne * D * D * D;
      if (precision == GBPA_F64X2) { ws_doubles += (size_t)d.ne * 6 * Q * Q * Q; }   // split qdata
      if (d.n_ess > 0) { mask_bytes += (size_t)d.ndofs; }
   }
   std::vector<int> gofs;
   if (graph)
   {
      const std::vector<char> all(nprob, 1);
      graph_tables(hp, groups, grp_of, all, batches, gofs, chunks);
   }
   // ---- device workspace: one allocation for everything
   const size_t nb = batches.size(), nc = chunks.size();
   size_t off = 0;
   auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
   const size_t o_probs = take(sizeof(BProb) * nprob);
   const size_t o_scal = take(sizeof(BScal) * nprob);
   const size_t o_batch = take(sizeof(BBatch) * (nb ? nb : 1));
   const size_t o_chunk = take(sizeof(BChunk) * (nc ? nc : 1));
   const size_t o_part = take(sizeof(double) * (nc ? nc : 1));
   const size_t o_sync = take(sizeof(unsigned int) * 64);
   const size_t o_cnt = take(sizeof(unsigned int) * nprob);
   const size_t o_ws = take(sizeof(double) * ws_doubles);
   const size_t o_mask = take(mask_bytes ? mask_bytes : 1);
   const size_t o_gm = take(sizeof(int) * (gm_ints ? gm_ints : 1));
   unsigned char *base = (unsigned char *)scratch(ctx, SLOT_BATCH, off);
   if (!base) { return GBPA_ERR_OUT_OF_MEMORY; }
   double *ws = (double *)(base + o_ws);
   unsigned char *mk = base + o_mask;
   int *gm = (int *)(base + o_gm);
   int rc = check_cuda(cudaMemsetAsync(base + o_sync, 0, sizeof(unsigned int) * 64, ctx->stream), "memset");
   if (!rc) { rc = check_cuda(cudaMemsetAsync(base + o_cnt, 0, sizeof(unsigned int) * nprob, ctx->stream), "memset"); }
   if (!rc && mask_bytes) { rc = check_cuda(cudaMemsetAsync(mk, 0, mask_bytes, ctx->stream), "memset"); }
   if (rc) { return rc; }
   for (int k = 0; k < nprob; ++k)
   {
      BProb &p = hp[k];
      const gbpa_problem_desc &d = probs[k];
      p.r = ws; p.d = ws + d.ndofs; p.z = ws + 2 * (size_t)d.ndofs; p.yE = ws + 3 * (size_t)d.ndofs;
      ws += 3 * (size_t)d.ndofs + (size_t)d.ne * d.d1d * d.d1d * d.d1d;
      p.qd2 = nullptr;
      if (precision == GBPA_F64X2)
      {
         const int64_t nq = (int64_t)d.ne * 6 * d.q1d * d.q1d * d.q1d;
         p.qd2 = (const float2 *)ws;
         rc = launch_split_x2(ctx, nq, d.qdata, (float2 *)ws);
         if (rc) { return rc; }
         ws += nq;
      }
      p.mask = nullptr;
      if (d.n_ess > 0)
      {
         batched_mask_kernel<<<grid_for(d.n_ess, 256), 256, 0, ctx->stream>>>(d.n_ess, d.ess, mk, d.ndofs,
                                                                            ctx->d_flags);
         rc = last_launch(ctx, "batched_mask");
         if (rc) { return rc; }
         p.mask = mk;
         mk += d.ndofs;
         // the element gather reads the pre-masked map (no mask lookup)
         const int64_t nE = (int64_t)d.ne * d.d1d * d.d1d * d.d1d;
         rc = launch_masked_gather_map(ctx, nE, d.gather_map, p.mask, gm);
         if (rc) { return rc; }
         p.gmap = gm;
         gm += nE;
      }
   }
   // initial solver state: problems without dofs are converged at iteration 0
   // (the other entries are set by the solve's first phase)
   std::vector<BScal> hs(nprob);
   for (int k = 0; k < nprob; ++k)
   {
      hs[k] = BScal{};
      if (hp[k].ndofs == 0) { hs[k].converged = 1; hs[k].done = 1; }
   }
   rc = check_cuda(cudaMemcpyAsync(base + o_probs, hp.data(), sizeof(BProb) * nprob, cudaMemcpyHostToDevice, ctx->stream), "copy");
   if (!rc) { rc = check_cuda(cudaMemcpyAsync(base + o_scal, hs.data(), sizeof(BScal) * nprob, cudaMemcpyHostToDevice, ctx->stream), "copy"); }
   if (!rc && nb) { rc = check_cuda(cudaMemcpyAsync(base + o_batch, batches.data(), sizeof(BBatch) * nb, cudaMemcpyHostToDevice, ctx->stream), "copy"); }
   if (!rc && nc) { rc = check_cuda(cudaMemcpyAsync(base + o_chunk, chunks.data(), sizeof(BChunk) * nc, cudaMemcpyHostToDevice, ctx->stream), "copy"); }
   if (rc) { return rc; }
   int flags0 = 0;
   rc = gbpa_get_error_flags(ctx, &flags0);   // syncs: host tables may change after
   if (rc) { return rc; }
   if (flags0 & GBPA_FLAG_INDEX) { return GBPA_ERR_INDEX; }

   float ms = 0.f;
   if (graph)
   {
      GParams G;
      G.probs = (const BProb *)(base + o_probs);
      G.scal = (BScal *)(base + o_scal);
      G.chunks = (const BChunk *)(base + o_chunk);
      G.partials = (double *)(base + o_part);
      G.cnt = (unsigned int *)(base + o_cnt);
      G.rel2 = rel_tol * rel_tol;
      G.abs2 = abs_tol * abs_tol;
      G.max_it = max_it;
      G.flags = ctx->d_flags;
      rc = run_graph_schedule(ctx, precision, hp, groups, grp_of, G, (BProb *)(base + o_probs),
                              (BBatch *)(base + o_batch), (BChunk *)(base + o_chunk), (int)nc, max_it, hs,
                              &ms);
      if (rc) { return rc; }
   }
   else
   {
      BParams P;
      P.probs = (const BProb *)(base + o_probs);
      P.scal = (BScal *)(base + o_scal);
      P.nprob = nprob;
      P.batches = (const BBatch *)(base + o_batch);
      P.nbatch = (int)nb;
      P.chunks = (const BChunk *)(base + o_chunk);
      P.nchunk = (int)nc;
      P.partials = (double *)(base + o_part);
      P.rel2 = rel_tol * rel_tol;
      P.abs2 = abs_tol * abs_tol;
      P.max_it = max_it;
      unsigned int *sync = (unsigned int *)(base + o_sync);
      P.bar_count = sync;
      P.bar_gen = sync + 32;
      P.flags = ctx->d_flags;
      P.n_active = (int *)(sync + 1);
      P.abort = (int *)(sync + 2);
      P.spin_limit = 1LL << 26;   // ~2 s of 32 ns sleeps

      const void *kfn = precision == GBPA_F64X2 ? (const void *)batched_pcg_kernel<ArX2>
                                                : (const void *)batched_pcg_kernel<ArF64>;
      rc = ensure_smem(kfn, smem_max);
      if (rc) { return rc; }
      int per_sm = 0;
      rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, BATCH_THREADS, smem_max),
                      "occupancy");
      if (rc) { return rc; }
      if (per_sm < 1) { return GBPA_ERR_UNSUPPORTED; }
      const int grid = per_sm * ctx->num_sms;
      void *args[] = {&P};
      StreamTimer timer(ctx->stream);
      rc = check_cuda(cudaLaunchCooperativeKernel(kfn, dim3(grid), dim3(BATCH_THREADS), args, smem_max,
                                                  ctx->stream), "cudaLaunchCooperativeKernel");
      ctx->launches++;
      if (!rc) { ms = timer.stop(ctx->stream); }
      if (rc) { return rc; }
      rc = check_cuda(cudaMemcpy(hs.data(), base + o_scal, sizeof(BScal) * nprob, cudaMemcpyDeviceToHost),
                      "copy back");
      if (rc) { return rc; }
   }
   if (seconds) { *seconds = ms * 1e-3; }
   int flags = 0;
   rc = gbpa_get_error_flags(ctx, &flags);
   if (rc) { return rc; }
   for (int k = 0; k < nprob; ++k)
   {
      if (iterations) { iterations[k] = hs[k].final_iter; }
      if (converged) { converged[k] = hs[k].converged; }
      if (final_norms) { final_norms[k] = hs[k].betanom >= 0 ? sqrt(hs[k].betanom) : hs[k].betanom; }
   }
   if (flags & GBPA_FLAG_TIMEOUT) { return GBPA_ERR_TIMEOUT; }
   if (flags & GBPA_FLAG_NOT_FINITE) { return GBPA_ERR_NOT_FINITE; }
   return GBPA_SUCCESS;
}
// ------------------------------------------------ bounded-wait self-test
// Each of the library's device waits is made to run out: the arrival it
// waits for never comes. The wait must give up after its limit, report
// GBPA_FLAG_TIMEOUT / a failed wait, and the kernel must return, leaving the
// context usable.
// (0) the persistent kernel's grid barrier, block 0 never arriving
__global__ void selftest_barrier_kernel(BParams P)
{
   if (blockIdx.x == 0) { return; }
   grid_barrier(P);
}
// (1) the TMA staging mbarrier wait, nothing arriving and no copy issued
__global__ void selftest_mbarrier_kernel(long long max_polls, int *timed_out)
{
   __shared__ unsigned long long bar;
   if (threadIdx.x == 0) { mbar_init(&bar, 1); }
   __syncthreads();
   const bool ok = mbar_wait(&bar, 0, max_polls);
   if (!ok && threadIdx.x == 0) { atomicOr(timed_out, GBPA_FLAG_TIMEOUT); }
}
} // namespace gbpa

using namespace gbpa;

extern "C" int gbpa_selftest_bounded_wait(gbpa_ctx_t ctx, int which, long long limit)
{
   if (!ctx || (which != 0 && which != 1) || limit < 1 || limit > (1LL << 26))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   unsigned int *sync = nullptr;
   int rc = check_cuda(cudaMalloc(&sync, 64 * sizeof(unsigned int)), "cudaMalloc");
   if (rc) { return rc; }
   rc = check_cuda(cudaMemsetAsync(sync, 0, 64 * sizeof(unsigned int), ctx->stream), "memset");
   if (!rc && which == 0)
   {
      BParams P{};
      P.bar_count = sync;
      P.bar_gen = sync + 32;
      P.abort = (int *)(sync + 2);
      P.flags = ctx->d_flags;
      P.spin_limit = limit;
      void *args[] = {&P};
      rc = check_cuda(cudaLaunchCooperativeKernel((const void *)selftest_barrier_kernel, dim3(2),
                                                  dim3(64), args, 0, ctx->stream),
                      "cudaLaunchCooperativeKernel");
      ctx->launches++;
   }
   else if (!rc)
   {
      selftest_mbarrier_kernel<<<1, 32, 0, ctx->stream>>>(limit, ctx->d_flags);
      rc = last_launch(ctx, "selftest_mbarrier");
   }
   if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "sync"); }
   cudaFree(sync);
   if (rc) { return rc; }
   int flags = 0;
   rc = gbpa_get_error_flags(ctx, &flags);
   if (rc) { return rc; }
   return (flags & GBPA_FLAG_TIMEOUT) ? GBPA_ERR_TIMEOUT : GBPA_SUCCESS;
}

extern "C" int gbpa_batched_pcg_solve_ex(gbpa_ctx_t ctx, int nprob, const gbpa_problem_desc *probs,
                                         int precision, int schedule, double rel_tol, double abs_tol,
                                         int max_it, int *iterations, int *converged, double *final_norms,
                                         double *seconds)
{
   return batched_solve(ctx, nprob, probs, precision, schedule, rel_tol, abs_tol, max_it, iterations,
                        converged, final_norms, seconds);
}

extern "C" int gbpa_batched_pcg_solve_precision(gbpa_ctx_t ctx, int nprob,
                                                const gbpa_problem_desc *probs, int precision,
                                                double rel_tol, double abs_tol, int max_it,
                                                int *iterations, int *converged,
                                                double *final_norms, double *seconds)
{
   return batched_solve(ctx, nprob, probs, precision, GBPA_BATCH_GRAPH, rel_tol, abs_tol, max_it,
                        iterations, converged, final_norms, seconds);
}

extern "C" int gbpa_batched_pcg_solve(gbpa_ctx_t ctx, int nprob, const gbpa_problem_desc *probs,
                                      double rel_tol, double abs_tol, int max_it, int *iterations,
                                      int *converged, double *final_norms, double *seconds)
{
   return batched_solve(ctx, nprob, probs, GBPA_F64, GBPA_BATCH_GRAPH, rel_tol, abs_tol, max_it,
                        iterations, converged, final_norms, seconds);
}
