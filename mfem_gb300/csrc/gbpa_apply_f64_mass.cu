// Native FP64 mass apply kernels.
#include "gbpa_apply_launch.cuh"

namespace gbpa
{
template <>
int launch_mass_apply<double>(gbpa_ctx *ctx, int ne, int D, int Q, const double *B,
                              const double *qd, const double *x, const int *gather_map,
                              const unsigned char *ess_mask, double *y, int accumulate,
                              const int *skip)
{
   return launch_mass_ar<ArF64>(ctx, GBPA_F64, ne, D, Q, B, qd, x, gather_map, ess_mask, y,
                                accumulate, skip);
}
} // namespace gbpa

namespace gbpa
{
int launch_mass_apply_qdiv(gbpa_ctx *ctx, int ne, int D, int Q, const double *B, const double *qd,
                           const double *x, double *y, int qdiv)
{
   return launch_mass_ar<ArF64>(ctx, GBPA_F64, ne, D, Q, B, qd, x, nullptr, nullptr, y, true, nullptr, qdiv);
}
} // namespace gbpa
