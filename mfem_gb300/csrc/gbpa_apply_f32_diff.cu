// Native FP32 diffusion apply kernels.
#include "gbpa_apply_launch.cuh"

namespace gbpa
{
template <>
int launch_diffusion_apply<float>(gbpa_ctx *ctx, int ne, int symm, int D, int Q,
                                  const float *B, const float *G, const float *qd,
                                  const float *x, const int *gather_map,
                                  const unsigned char *ess_mask, float *y, int accumulate,
                                  const int *skip)
{
   return launch_diffusion_ar<ArF32>(ctx, GBPA_F32, ne, symm, D, Q, B, G, qd, x, gather_map,
                                     ess_mask, y, accumulate, skip);
}
} // namespace gbpa
