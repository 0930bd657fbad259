// Native FP32 mass apply in the 3D thread layout (its own translation unit so that
// it compiles in parallel with the 2D-slab kernels).
#include "gbpa_apply_launch.cuh"

namespace gbpa
{
int launch_mass_3d_f32(gbpa_ctx *ctx, int ne, int D, int Q, const float *B, const float *qd, const float *x,
                       const int *gather_map, const unsigned char *ess_mask, float *y, int mode,
                       const int *skip, int nbz)
{
   return launch_mass_3d_ar<ArF32>(ctx, ne, D, Q, B, qd, x, gather_map, ess_mask, y, mode, skip, nbz);
}
} // namespace gbpa
