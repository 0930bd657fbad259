// FP64-accurate double-float mass apply kernels on the FP32
// pipes; FP64 inputs/outputs, qdata pre-split as float2 (hi, lo).
#include "gbpa_apply_launch.cuh"

namespace gbpa
{
int launch_mass_apply_x2(gbpa_ctx *ctx, int ne, int D, int Q, const double *B, const float2 *qd,
                         const double *x, const int *gather_map, const unsigned char *ess_mask,
                         double *y, int accumulate, const int *skip)
{
   return launch_mass_ar<ArX2, 10, false>(ctx, GBPA_F64X2, ne, D, Q, B, qd, x, gather_map, ess_mask, y,
                               accumulate, skip);
}

// qdata (FP64) -> (hi, lo) float pairs
__global__ void split_kernel(int64_t n, const double *__restrict__ a, float2 *__restrict__ b)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const double v = a[i];
      const float h = __double2float_rn(v);
      b[i] = make_float2(h, __double2float_rn(v - (double)h));
   }
}

int launch_split_x2(gbpa_ctx *ctx, int64_t n, const double *a, float2 *b)
{
   if (n == 0) { return GBPA_SUCCESS; }
   split_kernel<<<grid_for(n, 256, 16 * ctx->num_sms), 256, 0, ctx->stream>>>(n, a, b);
   return last_launch(ctx, "split_x2");
}
} // namespace gbpa
