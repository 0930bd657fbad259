// Grouped element apply of the batched PCG, native FP64 arithmetic.
#include "gbpa_batched_apply.cuh"

namespace gbpa
{
int batched_apply_nbz_f64(int D, int Q) { return batched_apply_nbz_ar<ArF64>(GBPA_F64, D, Q); }
int launch_batched_apply_f64(gbpa_ctx *ctx, int D, int Q, int nbz, const BBatch *batches, int nbatch,
                             const BProb *probs, const BScal *scal)
{
   return launch_batched_apply_ar<ArF64>(ctx, D, Q, nbz, batches, nbatch, probs, scal);
}
} // namespace gbpa
