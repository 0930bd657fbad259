// FP64-accurate double-float diffusion apply kernels on the FP32
// pipes; FP64 inputs/outputs, qdata pre-split as float2 (hi, lo).
#include "gbpa_apply_launch.cuh"

namespace gbpa
{
int launch_diffusion_apply_x2(gbpa_ctx *ctx, int ne, int symm, int D, int Q, const double *B,
                              const double *G, const float2 *qd, const double *x,
                              const int *gather_map, const unsigned char *ess_mask, double *y,
                              int accumulate, const int *skip)
{
   return launch_diffusion_ar<ArX2, 10, false>(ctx, GBPA_F64X2, ne, symm, D, Q, B, G, qd, x, gather_map,
                                    ess_mask, y, accumulate, skip);
}
} // namespace gbpa
