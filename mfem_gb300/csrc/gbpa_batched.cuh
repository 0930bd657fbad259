// Shared declarations of the batched PCG (many independent Dirichlet Poisson
// problems solved together): per-problem descriptors and solver scalars in
// device memory, work tables, and the grouped element-apply launcher used by
// the graph-captured schedule.
#pragma once
#include "gbpa_internal.cuh"

namespace gbpa
{
constexpr int BATCH_THREADS = 256;   // vector-phase blocks (and the persistent kernel)
constexpr int CHUNK = 2048;          // dofs per vector-phase block / partial sum

struct BProb
{
   int ne, ndofs, D, Q, nbz;
   const double *B, *G, *qd, *dinv, *b;
   const float2 *qd2;   // qdata split into (hi, lo) floats for the double-float arithmetic
   double *x;
   const int *gmap, *off, *ind;          // gmap: pre-masked (GBPA_GATHER_SKIP on ess slots) when mask is set
   const unsigned char *mask;           // ess mask (scatter), or null
   double *r, *d, *z, *yE;
   int chunk0, nchunk;
};
// Per-problem solver scalars (CGSolver::Mult's nom, den, betanom, alpha,
// beta and the iteration state).
struct BScal
{
   double nom, nom0, den, betanom, alpha, beta, r0;
   int iter, done, converged, final_iter;
};
// An element batch: count elements of problem `prob` from e0, one block.
struct BBatch { int prob, e0, count; };
// A dof chunk: dofs [i0, i1) of problem `prob`; its partial sum goes to
// partials[slot] (slot = the chunk's index in the problem's full chunk list).
struct BChunk { int prob, i0, i1, slot; };

// Elements per block of the grouped apply for (precision, D, Q): the tuned
// value clamped to the kernel's register-limited block size; 0 when the
// order is not supported.
int batched_apply_nbz(int precision, int D, int Q);
// One launch applying, for every batch in `batches` (all of one (D, Q) and
// blocks of nbz elements), yE = A_e d of the batch's problem, skipping
// problems whose scal.done is set. precision: GBPA_F64 or GBPA_F64X2.
int launch_batched_apply(gbpa_ctx *ctx, int precision, int D, int Q, int nbz, const BBatch *batches,
                         int nbatch, const BProb *probs, const BScal *scal);
} // namespace gbpa
