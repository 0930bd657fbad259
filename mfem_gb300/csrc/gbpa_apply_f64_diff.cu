// Native FP64 diffusion apply kernels.
#include "gbpa_apply_launch.cuh"

namespace gbpa
{
template <>
int launch_diffusion_apply<double>(gbpa_ctx *ctx, int ne, int symm, int D, int Q,
                                   const double *B, const double *G, const double *qd,
                                   const double *x, const int *gather_map,
                                   const unsigned char *ess_mask, double *y, int accumulate,
                                   const int *skip)
{
   return launch_diffusion_ar<ArF64>(ctx, GBPA_F64, ne, symm, D, Q, B, G, qd, x, gather_map,
                                     ess_mask, y, accumulate, skip);
}
} // namespace gbpa
