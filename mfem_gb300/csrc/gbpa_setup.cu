// Quadrature-data setup: geometric factors from the mesh nodes, diffusion
// and mass qdata, and the fused nodes -> qdata kernel.
//   geometric factors  mesh/mesh.cpp:15445-15500, fem/qinterp/grad.hpp:233-376,
//                      fem/qinterp/det.hpp:253-330, fem/qinterp/eval.hpp
//   diffusion setup    fem/integ/bilininteg_diffusion_kernels.cpp:262-386
//   mass setup         fem/integ/bilininteg_mass_pa.cpp:73-89
// One thread per (quadrature point, element); every kernel is FP64.
#include "gbpa_internal.cuh"

namespace gbpa
{

// J(c, d) = sum_{a} X(a, c) dphi_a/dxi_d at quadrature point (qx, qy, qz),
// evaluated directly from the 1D tables (a few dozen FMAs per entry for the
// order-1 and order-3 geometries used here).
__device__ void eval_jacobian(int dg, int Q, const double *__restrict__ Bg,
                              const double *__restrict__ Gg,
                              const double *__restrict__ Xe, int qx, int qy,
                              int qz, double J[3][3])
{
   const int D3 = dg * dg * dg;
#pragma unroll
   for (int c = 0; c < 3; ++c) { J[c][0] = J[c][1] = J[c][2] = 0.0; }
   for (int az = 0; az < dg; ++az)
   {
      const double bz = Bg[qz + Q * az], gz = Gg[qz + Q * az];
      for (int ay = 0; ay < dg; ++ay)
      {
         const double by = Bg[qy + Q * ay], gy = Gg[qy + Q * ay];
         for (int ax = 0; ax < dg; ++ax)
         {
            const double bx = Bg[qx + Q * ax], gx = Gg[qx + Q * ax];
            const int a = ax + dg * (ay + dg * az);
            const double w0 = gx * by * bz, w1 = bx * gy * bz, w2 = bx * by * gz;
#pragma unroll
            for (int c = 0; c < 3; ++c)
            {
               const double xv = Xe[a + D3 * c];
               J[c][0] += xv * w0;
               J[c][1] += xv * w1;
               J[c][2] += xv * w2;
            }
         }
      }
   }
}

__device__ __forceinline__ double det3(const double J[3][3])
{
   return J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) -
          J[1][0] * (J[0][1] * J[2][2] - J[2][1] * J[0][2]) +
          J[2][0] * (J[0][1] * J[1][2] - J[1][1] * J[0][2]);
}

// D = (W/detJ) adj(J) C adj(J)^T at one point; writes S entries with stride.
__device__ void diffusion_point(const double J[3][3], double w, int coeff_dim,
                                const double *__restrict__ C, long long cstride,
                                double *__restrict__ out, long long ostride)
{
   const double J11 = J[0][0], J21 = J[1][0], J31 = J[2][0];
   const double J12 = J[0][1], J22 = J[1][1], J32 = J[2][1];
   const double J13 = J[0][2], J23 = J[1][2], J33 = J[2][2];
   const double w_detJ = w / det3(J);
   const double A11 = (J22 * J33) - (J23 * J32);
   const double A12 = (J32 * J13) - (J12 * J33);
   const double A13 = (J12 * J23) - (J22 * J13);
   const double A21 = (J31 * J23) - (J21 * J33);
   const double A22 = (J11 * J33) - (J13 * J31);
   const double A23 = (J21 * J13) - (J11 * J23);
   const double A31 = (J21 * J32) - (J31 * J22);
   const double A32 = (J31 * J12) - (J11 * J32);
   const double A33 = (J11 * J22) - (J12 * J21);
   if (coeff_dim == 6 || coeff_dim == 9)
   {
      const bool sym = coeff_dim == 6;
      const double M11 = C[0], M12 = C[cstride], M13 = C[2 * cstride];
      const double M21 = sym ? M12 : C[3 * cstride];
      const double M22 = sym ? C[3 * cstride] : C[4 * cstride];
      const double M23 = sym ? C[4 * cstride] : C[5 * cstride];
      const double M31 = sym ? M13 : C[6 * cstride];
      const double M32 = sym ? M23 : C[7 * cstride];
      const double M33 = sym ? C[5 * cstride] : C[8 * cstride];
      const double R11 = M11 * A11 + M12 * A12 + M13 * A13;
      const double R12 = M11 * A21 + M12 * A22 + M13 * A23;
      const double R13 = M11 * A31 + M12 * A32 + M13 * A33;
      const double R21 = M21 * A11 + M22 * A12 + M23 * A13;
      const double R22 = M21 * A21 + M22 * A22 + M23 * A23;
      const double R23 = M21 * A31 + M22 * A32 + M23 * A33;
      const double R31 = M31 * A11 + M32 * A12 + M33 * A13;
      const double R32 = M31 * A21 + M32 * A22 + M33 * A23;
      const double R33 = M31 * A31 + M32 * A32 + M33 * A33;
      out[0] = w_detJ * (A11 * R11 + A12 * R21 + A13 * R31);
      out[ostride] = w_detJ * (A11 * R12 + A12 * R22 + A13 * R32);
      out[2 * ostride] = w_detJ * (A11 * R13 + A12 * R23 + A13 * R33);
      const double D22 = w_detJ * (A21 * R12 + A22 * R22 + A23 * R32);
      const double D23 = w_detJ * (A21 * R13 + A22 * R23 + A23 * R33);
      const double D33 = w_detJ * (A31 * R13 + A32 * R23 + A33 * R33);
      if (sym)
      {
         out[3 * ostride] = D22; out[4 * ostride] = D23; out[5 * ostride] = D33;
      }
      else
      {
         out[3 * ostride] = w_detJ * (A21 * R11 + A22 * R21 + A23 * R31);
         out[4 * ostride] = D22;
         out[5 * ostride] = D23;
         out[6 * ostride] = w_detJ * (A31 * R11 + A32 * R21 + A33 * R31);
         out[7 * ostride] = w_detJ * (A31 * R12 + A32 * R22 + A33 * R32);
         out[8 * ostride] = D33;
      }
   }
   else
   {
      const double C1 = C[0];
      const double C2 = coeff_dim == 3 ? C[cstride] : C1;
      const double C3 = coeff_dim == 3 ? C[2 * cstride] : C1;
      out[0] = w_detJ * (C1 * A11 * A11 + C2 * A12 * A12 + C3 * A13 * A13);
      out[ostride] = w_detJ * (C1 * A11 * A21 + C2 * A12 * A22 + C3 * A13 * A23);
      out[2 * ostride] = w_detJ * (C1 * A11 * A31 + C2 * A12 * A32 + C3 * A13 * A33);
      out[3 * ostride] = w_detJ * (C1 * A21 * A21 + C2 * A22 * A22 + C3 * A23 * A23);
      out[4 * ostride] = w_detJ * (C1 * A21 * A31 + C2 * A22 * A32 + C3 * A23 * A33);
      out[5 * ostride] = w_detJ * (C1 * A31 * A31 + C2 * A32 * A32 + C3 * A33 * A33);
   }
}

// mode: 0 = J, 1 = detJ, 2 = coordinates
__global__ void geom_kernel(int ne, int dg, int Q, const double *__restrict__ Bg,
                            const double *__restrict__ Gg,
                            const double *__restrict__ X, double *__restrict__ out,
                            int mode)
{
   const int Q3 = Q * Q * Q;
   const int64_t n = (int64_t)ne * Q3;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int q = (int)(i % Q3);
      const int64_t e = i / Q3;
      const int qx = q % Q, qy = (q / Q) % Q, qz = q / (Q * Q);
      const double *Xe = X + e * 3 * dg * dg * dg;
      if (mode == 2)
      {
         double xyz[3] = {0, 0, 0};
         for (int az = 0; az < dg; ++az)
            for (int ay = 0; ay < dg; ++ay)
               for (int ax = 0; ax < dg; ++ax)
               {
                  const double w = Bg[qx + Q * ax] * Bg[qy + Q * ay] * Bg[qz + Q * az];
                  const int a = ax + dg * (ay + dg * az);
                  for (int c = 0; c < 3; ++c) { xyz[c] += Xe[a + dg * dg * dg * c] * w; }
               }
         for (int c = 0; c < 3; ++c) { out[q + (int64_t)Q3 * (c + 3 * e)] = xyz[c]; }
         continue;
      }
      double J[3][3];
      eval_jacobian(dg, Q, Bg, Gg, Xe, qx, qy, qz, J);
      if (mode == 0)
      {
         for (int c = 0; c < 3; ++c)
            for (int d = 0; d < 3; ++d)
            {
               out[q + (int64_t)Q3 * (c + 3 * (d + 3 * e))] = J[c][d];
            }
      }
      else
      {
         out[q + (int64_t)Q3 * e] = det3(J);
      }
   }
}

__global__ void diffusion_setup_kernel(int ne, int Q3, int coeff_dim,
                                       const double *__restrict__ W,
                                       const double *__restrict__ Jg,
                                       const double *__restrict__ C, int const_c,
                                       double *__restrict__ D)
{
   const int S = coeff_dim == 9 ? 9 : 6;
   const int64_t n = (int64_t)ne * Q3;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int q = (int)(i % Q3);
      const int64_t e = i / Q3;
      double J[3][3];
      for (int c = 0; c < 3; ++c)
         for (int d = 0; d < 3; ++d) { J[c][d] = Jg[q + (int64_t)Q3 * (c + 3 * (d + 3 * e))]; }
      const double *Cp = const_c ? C : C + (int64_t)coeff_dim * i;
      diffusion_point(J, W[q], coeff_dim, Cp, 1, D + q + (int64_t)Q3 * S * e, Q3);
   }
}

// VectorDiffusionIntegrator::AssemblePA, 3D (fem/integ/bilininteg_vecdiffusion_pa.cpp:
// 213-276), scalar or vector coefficient: per component c the symmetric
// (W/detJ) adj(J) adj(J)^T scaled by C_k (k = c for a vector coefficient,
// 0 for a scalar one; C laid out (coeff_vdim, Q^3, NE)). Layout
// (Q^3, 6, vdim, NE): component c of element e is the scalar diffusion
// qdata of the pseudo-element c + vdim e, so the scalar apply runs on
// vdim NE pseudo-elements of the (D^3, vdim, NE) E-vector.
__global__ void vector_diffusion_setup_kernel(int ne, int Q3, int vdim, int coeff_vdim,
                                              const double *__restrict__ W,
                                              const double *__restrict__ Jg,
                                              const double *__restrict__ C, int const_c,
                                              double *__restrict__ D)
{
   const int64_t n = (int64_t)ne * Q3;
   const double one = 1.0;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int q = (int)(i % Q3);
      const int64_t e = i / Q3;
      double J[3][3];
      for (int c = 0; c < 3; ++c)
         for (int d = 0; d < 3; ++d) { J[c][d] = Jg[q + (int64_t)Q3 * (c + 3 * (d + 3 * e))]; }
      double d0[6];
      diffusion_point(J, W[q], 1, &one, 1, d0, 1);
      for (int c = 0; c < vdim; ++c)
      {
         const int k = coeff_vdim == 1 ? 0 : c;
         const double ck = const_c ? C[k] : C[k + (int64_t)coeff_vdim * i];
         double *out = D + q + (int64_t)Q3 * 6 * (c + (int64_t)vdim * e);
         for (int s = 0; s < 6; ++s) { out[(int64_t)s * Q3] = d0[s] * ck; }
      }
   }
}

// VectorDiffusionIntegrator::AssemblePA with a matrix coefficient (vdim = 3,
// fem/integ/bilininteg_vecdiffusion_pa.cpp:119-130,213-272): block b (0..8)
// holds the geometric 3x3 symmetric factor times the coefficient entry
// C(map[b]), map = {0,3,6,1,4,7,2,5,8}; block b = j + 3 i couples source
// component i into component j. Layout block-major (Q^3, 6, NE, 9), so each
// block is one scalar-diffusion qdata array (Q^3, 6, NE).
__global__ void vector_diffusion_setup_matrix_kernel(int ne, int Q3, const double *__restrict__ W,
                                                     const double *__restrict__ Jg,
                                                     const double *__restrict__ C, int const_c,
                                                     double *__restrict__ D)
{
   const int map[9] = {0, 3, 6, 1, 4, 7, 2, 5, 8};
   const int64_t n = (int64_t)ne * Q3;
   const double one = 1.0;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int q = (int)(i % Q3);
      const int64_t e = i / Q3;
      double J[3][3];
      for (int c = 0; c < 3; ++c)
         for (int d = 0; d < 3; ++d) { J[c][d] = Jg[q + (int64_t)Q3 * (c + 3 * (d + 3 * e))]; }
      double d0[6];
      diffusion_point(J, W[q], 1, &one, 1, d0, 1);
      for (int b = 0; b < 9; ++b)
      {
         const int k = map[b];
         const double ck = const_c ? C[k] : C[k + 9 * i];
         double *out = D + q + (int64_t)Q3 * 6 * (e + (int64_t)ne * b);
         for (int s = 0; s < 6; ++s) { out[(int64_t)s * Q3] = d0[s] * ck; }
      }
   }
}

// VectorMassIntegrator::AssemblePA with a matrix coefficient (vdim = 3,
// fem/integ/bilininteg_vecmass_pa.cpp:73-78,119-160): block b = 3 c + d holds
// C(b, q, e) W(q) detJ, coupling component d into component c. Layout
// block-major (Q^3, NE, 9): each block is one scalar-mass qdata array.
__global__ void vector_mass_setup_matrix_kernel(int ne, int Q3, const double *__restrict__ W,
                                                const double *__restrict__ Jg, const double *__restrict__ C,
                                                int const_c, double *__restrict__ D)
{
   const int64_t n = (int64_t)ne * Q3;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int q = (int)(i % Q3);
      const int64_t e = i / Q3;
      double J[3][3];
      for (int c = 0; c < 3; ++c)
         for (int d = 0; d < 3; ++d) { J[c][d] = Jg[q + (int64_t)Q3 * (c + 3 * (d + 3 * e))]; }
      const double w_det = W[q] * det3(J);
      for (int b = 0; b < 9; ++b)
      {
         const double cb = const_c ? C[b] : C[b + 9 * i];
         D[q + (int64_t)Q3 * (e + (int64_t)ne * b)] = cb * w_det;
      }
   }
}

// VectorMassIntegrator::AssemblePA, 3D (fem/integ/bilininteg_vecmass_pa.cpp:
// 119-160), scalar or vector coefficient: D(q, k, e) = C(k, q, e) W(q) detJ,
// layout (Q^3, coeff_vdim, NE).
__global__ void vector_mass_setup_kernel(int ne, int Q3, int coeff_vdim, const double *__restrict__ W,
                                         const double *__restrict__ Jg, const double *__restrict__ C,
                                         int const_c, double *__restrict__ D)
{
   const int64_t n = (int64_t)ne * Q3;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int q = (int)(i % Q3);
      const int64_t e = i / Q3;
      double J[3][3];
      for (int c = 0; c < 3; ++c)
         for (int d = 0; d < 3; ++d) { J[c][d] = Jg[q + (int64_t)Q3 * (c + 3 * (d + 3 * e))]; }
      const double w_det = W[q] * det3(J);
      for (int k = 0; k < coeff_vdim; ++k)
      {
         const double ck = const_c ? C[k] : C[k + (int64_t)coeff_vdim * i];
         D[q + (int64_t)Q3 * (k + (int64_t)coeff_vdim * e)] = ck * w_det;
      }
   }
}

__global__ void diffusion_setup_nodes_kernel(int ne, int dg, int Q, int coeff_dim,
                                             const double *__restrict__ W,
                                             const double *__restrict__ Bg,
                                             const double *__restrict__ Gg,
                                             const double *__restrict__ X,
                                             const double *__restrict__ C, int const_c,
                                             double *__restrict__ D)
{
   const int Q3 = Q * Q * Q;
   const int S = coeff_dim == 9 ? 9 : 6;
   const int64_t n = (int64_t)ne * Q3;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int q = (int)(i % Q3);
      const int64_t e = i / Q3;
      double J[3][3];
      eval_jacobian(dg, Q, Bg, Gg, X + e * 3 * dg * dg * dg, q % Q, (q / Q) % Q, q / (Q * Q), J);
      const double *Cp = const_c ? C : C + (int64_t)coeff_dim * i;
      diffusion_point(J, W[q], coeff_dim, Cp, 1, D + q + (int64_t)Q3 * S * e, Q3);
   }
}

__global__ void mass_setup_kernel(int ne, int nq, const double *__restrict__ W,
                                  const double *__restrict__ detJ,
                                  const double *__restrict__ C, int const_c,
                                  int by_val, double *__restrict__ D)
{
   const int64_t n = (int64_t)ne * nq;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const double dj = detJ[i];
      const double c = const_c ? C[0] : C[i];
      D[i] = W[i % nq] * c * (by_val ? dj : 1.0 / dj);
   }
}

} // namespace gbpa

using namespace gbpa;

static int geom_common(gbpa_ctx_t ctx, int ne, int dg, int q1d, const double *Bg,
                       const double *Gg, const double *X, double *out, int mode)
{
   if (!ctx || ne < 0 || dg < 1 || q1d < 1 || dg > GBPA_MAX_1D || q1d > GBPA_MAX_1D)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (ne == 0) { return GBPA_SUCCESS; }
   if (!Bg || !X || !out || (mode != 2 && !Gg)) { return GBPA_ERR_INVALID_ARGUMENT; }
   const int64_t n = (int64_t)ne * q1d * q1d * q1d;
   geom_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(ne, dg, q1d, Bg, Gg, X, out, mode);
   return last_launch(ctx, "geom");
}

extern "C" int gbpa_geom_jacobians3d(gbpa_ctx_t ctx, int ne, int dg, int q1d,
                                     const double *Bg, const double *Gg, const double *X,
                                     double *J)
{
   return geom_common(ctx, ne, dg, q1d, Bg, Gg, X, J, 0);
}

extern "C" int gbpa_geom_determinants3d(gbpa_ctx_t ctx, int ne, int dg, int q1d,
                                        const double *Bg, const double *Gg, const double *X,
                                        double *detJ)
{
   return geom_common(ctx, ne, dg, q1d, Bg, Gg, X, detJ, 1);
}

extern "C" int gbpa_geom_coordinates3d(gbpa_ctx_t ctx, int ne, int dg, int q1d,
                                       const double *Bg, const double *X, double *XQ)
{
   return geom_common(ctx, ne, dg, q1d, Bg, nullptr, X, XQ, 2);
}

// Fourier modes of the lognormal coefficient, passed by value (kernel
// parameter space, read through the constant cache: every thread reads the
// same mode at the same time).
struct LognormalModes
{
   int n;
   double amp;
   double k[GBPA_MAX_MODES][3];
   double phi[GBPA_MAX_MODES];
};

// out(q, e) = exp(sum_m amp cos(2 pi k_m . x(q, e) + phi_m)), x from the
// (Q^3, 3, NE) coordinates array.
__global__ void lognormal_kernel(int64_t npts, int nq, const double *__restrict__ XQ,
                                 const __grid_constant__ LognormalModes modes,
                                 double *__restrict__ out)
{
   const double two_pi = 6.283185307179586476925286766559;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int64_t e = i / nq, q = i - e * nq;
      const double *xe = XQ + e * 3 * nq + q;
      const double x = xe[0], y = xe[nq], z = xe[2 * nq];
      double g = 0.0;
      for (int m = 0; m < modes.n; ++m)
      {
         const double a = two_pi * (modes.k[m][0] * x + modes.k[m][1] * y + modes.k[m][2] * z) + modes.phi[m];
         g += modes.amp * cos(a);
      }
      out[i] = exp(g);
   }
}

extern "C" int gbpa_coefficient_lognormal3d(gbpa_ctx_t ctx, int ne, int nq, const double *XQ,
                                            int nmodes, const int *k, const double *phi, double amp,
                                            double *out)
{
   if (!ctx || ne < 0 || nq < 1 || nmodes < 0 || nmodes > GBPA_MAX_MODES) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (ne == 0) { return GBPA_SUCCESS; }
   if (!XQ || !out || (nmodes > 0 && (!k || !phi))) { return GBPA_ERR_INVALID_ARGUMENT; }
   LognormalModes m{};
   m.n = nmodes;
   m.amp = amp;
   for (int i = 0; i < nmodes; ++i)
   {
      for (int d = 0; d < 3; ++d) { m.k[i][d] = (double)k[3 * i + d]; }
      m.phi[i] = phi[i];
   }
   const int64_t n = (int64_t)ne * nq;
   lognormal_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, nq, XQ, m, out);
   return last_launch(ctx, "coefficient_lognormal");
}

static int coeff_ok(int coeff_dim, int64_t c_size, int64_t npts)
{
   if (coeff_dim != 1 && coeff_dim != 3 && coeff_dim != 6 && coeff_dim != 9) { return 0; }
   return c_size == coeff_dim || c_size == coeff_dim * npts;
}

extern "C" int gbpa_diffusion_setup3d(gbpa_ctx_t ctx, int ne, int q1d, int coeff_dim,
                                      const double *W, const double *J, const double *C,
                                      int64_t c_size, double *D)
{
   if (!ctx || ne < 0 || q1d < 1 || q1d > GBPA_MAX_1D) { return GBPA_ERR_INVALID_ARGUMENT; }
   const int Q3 = q1d * q1d * q1d;
   if (!coeff_ok(coeff_dim, c_size, (int64_t)ne * Q3)) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (ne == 0) { return GBPA_SUCCESS; }
   if (!W || !J || !C || !D) { return GBPA_ERR_INVALID_ARGUMENT; }
   const int64_t n = (int64_t)ne * Q3;
   diffusion_setup_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(
      ne, Q3, coeff_dim, W, J, C, c_size == coeff_dim ? 1 : 0, D);
   return last_launch(ctx, "diffusion_setup");
}

extern "C" int gbpa_diffusion_setup3d_nodes(gbpa_ctx_t ctx, int ne, int dg, int q1d,
                                            int coeff_dim, const double *W, const double *Bg,
                                            const double *Gg, const double *X, const double *C,
                                            int64_t c_size, double *D)
{
   if (!ctx || ne < 0 || q1d < 1 || q1d > GBPA_MAX_1D || dg < 1 || dg > GBPA_MAX_1D)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   const int Q3 = q1d * q1d * q1d;
   if (!coeff_ok(coeff_dim, c_size, (int64_t)ne * Q3)) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (ne == 0) { return GBPA_SUCCESS; }
   if (!W || !Bg || !Gg || !X || !C || !D) { return GBPA_ERR_INVALID_ARGUMENT; }
   const int64_t n = (int64_t)ne * Q3;
   diffusion_setup_nodes_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(
      ne, dg, q1d, coeff_dim, W, Bg, Gg, X, C, c_size == coeff_dim ? 1 : 0, D);
   return last_launch(ctx, "diffusion_setup_nodes");
}

extern "C" int gbpa_mass_setup3d(gbpa_ctx_t ctx, int ne, int nq, const double *W,
                                 const double *detJ, const double *C, int64_t c_size,
                                 int by_val, double *D)
{
   if (!ctx || ne < 0 || nq < 1) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (c_size != 1 && c_size != (int64_t)ne * nq) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (ne == 0) { return GBPA_SUCCESS; }
   if (!W || !detJ || !C || !D) { return GBPA_ERR_INVALID_ARGUMENT; }
   const int64_t n = (int64_t)ne * nq;
   mass_setup_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(ne, nq, W, detJ, C,
                                                                c_size == 1 ? 1 : 0,
                                                                by_val ? 1 : 0, D);
   return last_launch(ctx, "mass_setup");
}

extern "C" int gbpa_vector_diffusion_setup3d(gbpa_ctx_t ctx, int ne, int q1d, int vdim, int coeff_vdim,
                                             const double *W, const double *J, const double *C, int64_t c_size,
                                             double *D)
{
   const bool matrix = vdim == 3 && coeff_vdim == 9;
   if (!ctx || ne < 0 || q1d < 1 || vdim < 1 || vdim > 3 || (coeff_vdim != 1 && coeff_vdim != vdim && !matrix))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   const int Q3 = q1d * q1d * q1d;
   if (c_size != coeff_vdim && c_size != (int64_t)coeff_vdim * ne * Q3) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (ne == 0) { return GBPA_SUCCESS; }
   if (!W || !J || !C || !D) { return GBPA_ERR_INVALID_ARGUMENT; }
   const int64_t n = (int64_t)ne * Q3;
   if (matrix)
   {
      vector_diffusion_setup_matrix_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(ne, Q3, W, J, C,
                                                                                     c_size == 9 ? 1 : 0, D);
      return last_launch(ctx, "vector_diffusion_setup_matrix");
   }
   vector_diffusion_setup_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(ne, Q3, vdim, coeff_vdim, W, J, C,
                                                                            c_size == coeff_vdim ? 1 : 0, D);
   return last_launch(ctx, "vector_diffusion_setup");
}

extern "C" int gbpa_vector_mass_setup3d(gbpa_ctx_t ctx, int ne, int q1d, int vdim, int coeff_vdim, const double *W,
                                        const double *J, const double *C, int64_t c_size, double *D)
{
   const bool matrix = vdim == 3 && coeff_vdim == 9;
   if (!ctx || ne < 0 || q1d < 1 || vdim < 1 || vdim > 3 || (coeff_vdim != 1 && coeff_vdim != vdim && !matrix))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   const int Q3 = q1d * q1d * q1d;
   if (c_size != coeff_vdim && c_size != (int64_t)coeff_vdim * ne * Q3) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (ne == 0) { return GBPA_SUCCESS; }
   if (!W || !J || !C || !D) { return GBPA_ERR_INVALID_ARGUMENT; }
   const int64_t n = (int64_t)ne * Q3;
   if (matrix)
   {
      vector_mass_setup_matrix_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(ne, Q3, W, J, C,
                                                                                c_size == 9 ? 1 : 0, D);
      return last_launch(ctx, "vector_mass_setup_matrix");
   }
   vector_mass_setup_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(ne, Q3, coeff_vdim, W, J, C,
                                                                       c_size == coeff_vdim ? 1 : 0, D);
   return last_launch(ctx, "vector_mass_setup");
}
