// Grouped element apply of the batched PCG, double-float arithmetic on the
// FP32 pipes (qdata pre-split into float2 (hi, lo)).
#include "gbpa_batched_apply.cuh"

namespace gbpa
{
int batched_apply_nbz_x2(int D, int Q) { return batched_apply_nbz_ar<ArX2>(GBPA_F64X2, D, Q); }
int launch_batched_apply_x2(gbpa_ctx *ctx, int D, int Q, int nbz, const BBatch *batches, int nbatch,
                            const BProb *probs, const BScal *scal)
{
   return launch_batched_apply_ar<ArX2>(ctx, D, Q, nbz, batches, nbatch, probs, scal);
}
} // namespace gbpa
