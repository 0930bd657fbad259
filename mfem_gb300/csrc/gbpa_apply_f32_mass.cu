// Native FP32 mass apply kernels.
#include "gbpa_apply_launch.cuh"

namespace gbpa
{
template <>
int launch_mass_apply<float>(gbpa_ctx *ctx, int ne, int D, int Q, const float *B,
                             const float *qd, const float *x, const int *gather_map,
                             const unsigned char *ess_mask, float *y, int accumulate,
                             const int *skip)
{
   return launch_mass_ar<ArF32>(ctx, GBPA_F32, ne, D, Q, B, qd, x, gather_map, ess_mask, y,
                                accumulate, skip);
}
} // namespace gbpa
