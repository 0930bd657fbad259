// Native FP32 block (several right-hand sides) diffusion apply kernels, in their own
// translation unit so that they compile in parallel with the single-vector ones.
#include "gbpa_apply_launch.cuh"

namespace gbpa
{
int launch_diffusion_block_f32(gbpa_ctx *ctx, int ne, int nrhs, int symm, int D, int Q,
                               const float *B, const float *G, const float *qd, const float *x,
                               const int *gather_map, const unsigned char *ess_mask, float *y,
                               const int *skip)
{
   return launch_diffusion_block_ar<ArF32>(ctx, ne, nrhs, symm, D, Q, B, G, qd, x, gather_map,
                                           ess_mask, y, skip);
}
} // namespace gbpa
