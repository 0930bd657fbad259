// Vector diffusion and vector mass PA with a matrix coefficient (vdim = 3):
// the coefficient couples the components, y_j += sum_i A_{b(i,j)} x_i, with
// A_b the scalar operator of coefficient block b. The E-vectors (D^3, 3, NE)
// are permuted to component-major (D^3, NE, 3) in scratch, the nine blocks run
// as scalar E-vector applies (each reads one block-major qdata array written
// by the matrix setups in gbpa_setup.cu), and the result is added back in the
// reference's layout. Reference: fem/integ/bilininteg_vecdiffusion_pa.hpp:
// 96-163 (block j + 3 i for source i, destination j) and
// fem/integ/bilininteg_vecmass_pa.hpp:157-170 (block 3 c + d for source d,
// destination c).
#include "gbpa_dispatch.cuh"

namespace
{
// out[(c NE + e) nd + i] = in[(e 3 + c) nd + i]
__global__ void to_component_major(int64_t n, int ne, int nd, const double *__restrict__ in,
                                   double *__restrict__ out)
{
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      const int i = (int)(k % nd);
      const int64_t ec = k / nd;
      const int c = (int)(ec % 3);
      const int64_t e = ec / 3;
      out[((int64_t)c * ne + e) * nd + i] = in[k];
   }
}

// y[(e 3 + c) nd + i] += t[(c NE + e) nd + i]
__global__ void add_from_component_major(int64_t n, int ne, int nd, const double *__restrict__ t,
                                         double *__restrict__ y)
{
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      const int i = (int)(k % nd);
      const int64_t ec = k / nd;
      const int c = (int)(ec % 3);
      const int64_t e = ec / 3;
      y[k] += t[((int64_t)c * ne + e) * nd + i];
   }
}

bool dq_ok(int D, int Q) { return D >= 1 && Q >= 1 && D <= GBPA_MAX_1D && Q <= GBPA_MAX_1D; }

// kind 0: diffusion (block of source i, destination j = j + 3 i; qdata block
// stride 6 Q^3 NE); kind 1: mass (block 3 j + i; stride Q^3 NE)
int coupled_apply(gbpa_ctx *ctx, int kind, int ne, int D, int Q, const double *B, const double *G,
                  const double *qd, const double *x, double *y)
{
   const int nd = D * D * D;
   const int64_t n = (int64_t)3 * ne * nd;
   double *xp = (double *)gbpa::scratch(ctx, gbpa::SLOT_TMP, sizeof(double) * 2 * (size_t)n);
   if (!xp) { return GBPA_ERR_OUT_OF_MEMORY; }
   double *yp = xp + n;
   const unsigned g = gbpa::grid_for(n, 256, 8 * ctx->num_sms);
   to_component_major<<<g, 256, 0, ctx->stream>>>(n, ne, nd, x, xp);
   int rc = gbpa::last_launch(ctx, "to_component_major");
   if (!rc) { rc = gbpa::check_cuda(cudaMemsetAsync(yp, 0, sizeof(double) * n, ctx->stream), "memset"); }
   const int64_t Q3 = (int64_t)Q * Q * Q;
   const int64_t qstride = (kind == 0 ? 6 : 1) * Q3 * ne;
   for (int i = 0; i < 3 && !rc; ++i)
   {
      for (int j = 0; j < 3 && !rc; ++j)
      {
         const int b = kind == 0 ? j + 3 * i : 3 * j + i;
         const double *xi = xp + (int64_t)i * ne * nd;
         double *yj = yp + (int64_t)j * ne * nd;
         rc = kind == 0 ? gbpa::launch_diffusion_apply<double>(ctx, ne, 1, D, Q, B, G, qd + b * qstride, xi,
                                                               nullptr, nullptr, yj, 1)
                        : gbpa::launch_mass_apply<double>(ctx, ne, D, Q, B, qd + b * qstride, xi, nullptr,
                                                          nullptr, yj, 1);
      }
   }
   if (!rc)
   {
      add_from_component_major<<<g, 256, 0, ctx->stream>>>(n, ne, nd, yp, y);
      rc = gbpa::last_launch(ctx, "add_from_component_major");
   }
   return rc;
}
} // namespace

extern "C" int gbpa_vector_diffusion_apply3d_coeff(gbpa_ctx_t ctx, int ne, int vdim, int coeff_vdim, int d1d,
                                                   int q1d, const double *B, const double *G, const double *D,
                                                   const double *x, double *y)
{
   if (!ctx || ne < 0 || vdim < 1 || vdim > 3) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (coeff_vdim == 1 || coeff_vdim == vdim)
   {
      return gbpa_vector_diffusion_apply3d(ctx, ne, vdim, d1d, q1d, B, G, D, x, y);
   }
   if (vdim != 3 || coeff_vdim != 9) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (ne > 0 && (!B || !G || !D || !x || !y)) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (!dq_ok(d1d, q1d)) { return GBPA_ERR_UNSUPPORTED; }
   if (ne == 0) { return GBPA_SUCCESS; }
   return coupled_apply(ctx, 0, ne, d1d, q1d, B, G, D, x, y);
}

namespace gbpa
{
int vector_mass_apply_matrix(gbpa_ctx *ctx, int ne, int d1d, int q1d, const double *B, const double *D,
                             const double *x, double *y)
{
   if (ne == 0) { return GBPA_SUCCESS; }
   return coupled_apply(ctx, 1, ne, d1d, q1d, B, nullptr, D, x, y);
}
} // namespace gbpa
