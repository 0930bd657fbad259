// Native FP64 block (several right-hand sides) diffusion apply kernels, in their own
// translation unit so that they compile in parallel with the single-vector ones.
#include "gbpa_apply_launch.cuh"

namespace gbpa
{
int launch_diffusion_block_f64(gbpa_ctx *ctx, int ne, int nrhs, int symm, int D, int Q,
                               const double *B, const double *G, const double *qd, const double *x,
                               const int *gather_map, const unsigned char *ess_mask, double *y,
                               const int *skip)
{
   return launch_diffusion_block_ar<ArF64>(ctx, ne, nrhs, symm, D, Q, B, G, qd, x, gather_map,
                                           ess_mask, y, skip);
}
} // namespace gbpa
