/* CPU oracle for the partial-assembly H1 path (test infrastructure only).
 * A plain-C restatement of the reference algorithms named in gbpa_oracle.h;
 * only tests/, smoke() and bench.py's CPU-baseline leg load it, as the checker.
 * Element loops run under OpenMP when built with -fopenmp, which changes no
 * result: every output entry is produced by exactly one thread in a fixed
 * summation order. */
#define _USE_MATH_DEFINES
#include "gbpa_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAXQ 16
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int or_num_threads(void)
{
#ifdef _OPENMP
   return omp_get_max_threads();
#else
   return 1;
#endif
}

void or_set_num_threads(int n)
{
#ifdef _OPENMP
   if (n > 0) { omp_set_num_threads(n); }
#else
   (void)n;
#endif
}

/* ------------------------------------------------------------ restriction */
void or_restriction_build(int ne, int dof, int ndofs, const int *elem_dofs,
                          const int *dof_map, int *offsets, int *indices,
                          int *gather_map)
{
   /* fem/restriction.cpp:72-113: count multiplicities, prefix-sum, fill the
    * CSR rows in element order, then shift the offsets back by one. */
   for (int i = 0; i <= ndofs; ++i) { offsets[i] = 0; }
   for (int e = 0; e < ne; ++e)
      for (int d = 0; d < dof; ++d)
      {
         const int sgid = elem_dofs[dof * e + d];
         const int gid = sgid >= 0 ? sgid : -1 - sgid;
         ++offsets[gid + 1];
      }
   for (int i = 1; i <= ndofs; ++i) { offsets[i] += offsets[i - 1]; }
   for (int e = 0; e < ne; ++e)
      for (int d = 0; d < dof; ++d)
      {
         const int sdid = dof_map ? dof_map[d] : 0;
         const int did = !dof_map ? d : (sdid >= 0 ? sdid : -1 - sdid);
         const int sgid = elem_dofs[dof * e + did];
         const int gid = sgid >= 0 ? sgid : -1 - sgid;
         const int lid = dof * e + d;
         const int plus = (sgid >= 0 && sdid >= 0) || (sgid < 0 && sdid < 0);
         gather_map[lid] = plus ? gid : -1 - gid;
         indices[offsets[gid]++] = plus ? lid : -1 - lid;
      }
   for (int i = ndofs; i > 0; --i) { offsets[i] = offsets[i - 1]; }
   offsets[0] = 0;
}

void or_restriction_mult(int ne, int nd, const int *gather_map,
                         const double *x, double *y)
{
   const long n = (long)ne * nd;
#pragma omp parallel for schedule(static)
   for (long i = 0; i < n; ++i)
   {
      const int gid = gather_map[i];
      const int j = gid >= 0 ? gid : -1 - gid;
      y[i] = gid >= 0 ? x[j] : -x[j];
   }
}

void or_restriction_mult_transpose(int nd, int ndofs, const int *offsets,
                                   const int *indices, const double *x,
                                   double *y, int add)
{
   (void)nd;
#pragma omp parallel for schedule(static)
   for (int i = 0; i < ndofs; ++i)
   {
      double v = 0.0;
      for (int j = offsets[i]; j < offsets[i + 1]; ++j)
      {
         const int s = indices[j];
         const int k = s >= 0 ? s : -1 - s;
         v += s >= 0 ? x[k] : -x[k];
      }
      if (add) { y[i] += v; } else { y[i] = v; }
   }
}

void or_restriction_abs_mult_transpose(int nd, int ndofs, const int *offsets,
                                       const int *indices, const double *x,
                                       double *y)
{
   (void)nd;
#pragma omp parallel for schedule(static)
   for (int i = 0; i < ndofs; ++i)
   {
      double v = 0.0;
      for (int j = offsets[i]; j < offsets[i + 1]; ++j)
      {
         const int s = indices[j];
         v += x[s >= 0 ? s : -1 - s];
      }
      y[i] = v;
   }
}

/* ------------------------------------------------------- quadrature/basis */
static void legendre(int n, double z, double *pn, double *pnm1)
{
   double p0 = 1.0, p1 = z;
   if (n == 0) { *pn = 1.0; *pnm1 = 0.0; return; }
   for (int j = 2; j <= n; ++j)
   {
      const double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j;
      p0 = p1; p1 = p2;
   }
   *pn = p1; *pnm1 = p0;
}

void or_gauss_legendre(int n, double *x, double *w)
{
   /* Newton iteration on P_n from the Chebyshev-like initial guess
    * cos(pi (i - 1/4) / (n + 1/2)), mapped to [0,1] (fem/intrules.cpp:642-690) */
   const int m = (n + 1) / 2;
   for (int i = 1; i <= m; ++i)
   {
      double z = cos(M_PI * (i - 0.25) / (n + 0.5));
      double pn, pm, pp, xi = 0.0;
      int done = 0;
      for (;;)
      {
         legendre(n, z, &pn, &pm);
         pp = n * (z * pn - pm) / (z * z - 1);
         if (done) { break; }
         const double dz = pn / pp;
         if (fabs(dz) < 1e-16)
         {
            done = 1;
            xi = ((1 - z) + dz) / 2;
         }
         z -= dz;
      }
      x[i - 1] = xi;
      x[n - i] = 1 - xi;
      w[i - 1] = w[n - i] = 1.0 / (4 * xi * (1 - xi) * pp * pp);
   }
}

void or_gauss_lobatto(int n, double *x)
{
   /* Interior points: zeros of P'_{n-1}, Newton from the Chebyshev-Lobatto
    * guess, symmetric halves (fem/intrules.cpp:708-800). */
   x[0] = 0.0;
   if (n == 1) { x[0] = 0.5; return; }
   x[n - 1] = 1.0;
   const int N = n - 1;
   for (int i = 1; i <= (n - 1) / 2; ++i)
   {
      double z = sin(M_PI * ((double)i / N - 0.5));
      for (int it = 0; it < 100; ++it)
      {
         double pn, pm;
         legendre(N, z, &pn, &pm);
         const double dp = N * (z * pn - pm) / (z * z - 1);           /* P'_N  */
         const double d2p = (2 * z * dp - N * (N + 1) * pn) / (1 - z * z); /* P''_N */
         const double dz = dp / d2p;
         z -= dz;
         if (fabs(dz) < 1e-16) { break; }
      }
      x[i] = (1.0 + z) / 2.0;
      x[n - 1 - i] = 1.0 - x[i];
   }
   if (n % 2 == 1) { x[n / 2] = 0.5; }
}

void or_basis_tables(int D, const double *nodes, int Q, const double *xq,
                     double *B, double *G)
{
   for (int q = 0; q < Q; ++q)
   {
      const double y = xq[q];
      for (int j = 0; j < D; ++j)
      {
         double v = 1.0, dv = 0.0;
         for (int m = 0; m < D; ++m)
         {
            if (m == j) { continue; }
            const double den = nodes[j] - nodes[m];
            /* product rule: d/dy prod (y-x_m)/den */
            dv = dv * (y - nodes[m]) / den + v / den;
            v = v * (y - nodes[m]) / den;
         }
         B[q + Q * j] = v;
         G[q + Q * j] = dv;
      }
   }
}

/* --------------------------------------------------- geometric factors */
void or_geom_jacobians3d(int ne, int dg, int q1d, const double *Bg,
                         const double *Gg, const double *X, double *J)
{
   const int D = dg, Q = q1d, Q3 = Q * Q * Q, D3 = D * D * D;
#pragma omp parallel for schedule(static)
   for (int e = 0; e < ne; ++e)
   {
      double DDQ0[OR_MAXQ][OR_MAXQ][OR_MAXQ], DDQ1[OR_MAXQ][OR_MAXQ][OR_MAXQ];
      double DQQ0[OR_MAXQ][OR_MAXQ][OR_MAXQ], DQQ1[OR_MAXQ][OR_MAXQ][OR_MAXQ],
             DQQ2[OR_MAXQ][OR_MAXQ][OR_MAXQ];
      for (int c = 0; c < 3; ++c)
      {
         const double *x = X + (long)D3 * (c + 3L * e);
         for (int dz = 0; dz < D; ++dz)
            for (int dy = 0; dy < D; ++dy)
               for (int qx = 0; qx < Q; ++qx)
               {
                  double u = 0.0, v = 0.0;
                  for (int dx = 0; dx < D; ++dx)
                  {
                     const double in = x[dx + D * (dy + D * dz)];
                     u += in * Bg[qx + Q * dx];
                     v += in * Gg[qx + Q * dx];
                  }
                  DDQ0[dz][dy][qx] = u; DDQ1[dz][dy][qx] = v;
               }
         for (int dz = 0; dz < D; ++dz)
            for (int qy = 0; qy < Q; ++qy)
               for (int qx = 0; qx < Q; ++qx)
               {
                  double u = 0.0, v = 0.0, w = 0.0;
                  for (int dy = 0; dy < D; ++dy)
                  {
                     u += DDQ1[dz][dy][qx] * Bg[qy + Q * dy];
                     v += DDQ0[dz][dy][qx] * Gg[qy + Q * dy];
                     w += DDQ0[dz][dy][qx] * Bg[qy + Q * dy];
                  }
                  DQQ0[dz][qy][qx] = u; DQQ1[dz][qy][qx] = v; DQQ2[dz][qy][qx] = w;
               }
         for (int qz = 0; qz < Q; ++qz)
            for (int qy = 0; qy < Q; ++qy)
               for (int qx = 0; qx < Q; ++qx)
               {
                  double u = 0.0, v = 0.0, w = 0.0;
                  for (int dz = 0; dz < D; ++dz)
                  {
                     u += DQQ0[dz][qy][qx] * Bg[qz + Q * dz];
                     v += DQQ1[dz][qy][qx] * Bg[qz + Q * dz];
                     w += DQQ2[dz][qy][qx] * Gg[qz + Q * dz];
                  }
                  const long q = qx + Q * (qy + Q * qz);
                  J[q + Q3 * (c + 3L * (0 + 3L * e))] = u;
                  J[q + Q3 * (c + 3L * (1 + 3L * e))] = v;
                  J[q + Q3 * (c + 3L * (2 + 3L * e))] = w;
               }
      }
   }
}

void or_geom_det3d(int ne, const double *J, int q3, double *detJ)
{
#pragma omp parallel for schedule(static)
   for (int e = 0; e < ne; ++e)
      for (int q = 0; q < q3; ++q)
      {
#define JJ(r, c) J[q + (long)q3 * ((r) + 3L * ((c) + 3L * e))]
         const double J11 = JJ(0, 0), J21 = JJ(1, 0), J31 = JJ(2, 0);
         const double J12 = JJ(0, 1), J22 = JJ(1, 1), J32 = JJ(2, 1);
         const double J13 = JJ(0, 2), J23 = JJ(1, 2), J33 = JJ(2, 2);
#undef JJ
         detJ[q + (long)q3 * e] = J11 * (J22 * J33 - J32 * J23) -
                                  J21 * (J12 * J33 - J32 * J13) +
                                  J31 * (J12 * J23 - J22 * J13);
      }
}

/* ---------------------------------------------------------- diffusion */
void or_diffusion_setup3d(int ne, int q1d, int coeff_dim, const double *W,
                          const double *J, const double *C, long c_size,
                          double *Dq)
{
   const int Q3 = q1d * q1d * q1d;
   const int symmetric = coeff_dim != 9;
   const int S = symmetric ? 6 : 9;
   const int const_c = c_size == coeff_dim;
#pragma omp parallel for schedule(static)
   for (int e = 0; e < ne; ++e)
      for (int q = 0; q < Q3; ++q)
      {
#define JJ(r, c) J[q + (long)Q3 * ((r) + 3L * ((c) + 3L * e))]
#define CC(i) (const_c ? C[i] : C[(i) + (long)coeff_dim * (q + (long)Q3 * e)])
#define DD(k) Dq[q + (long)Q3 * ((k) + (long)S * e)]
         const double J11 = JJ(0, 0), J21 = JJ(1, 0), J31 = JJ(2, 0);
         const double J12 = JJ(0, 1), J22 = JJ(1, 1), J32 = JJ(2, 1);
         const double J13 = JJ(0, 2), J23 = JJ(1, 2), J33 = JJ(2, 2);
         const double detJ = J11 * (J22 * J33 - J32 * J23) -
                             J21 * (J12 * J33 - J32 * J13) +
                             J31 * (J12 * J23 - J22 * J13);
         const double w_detJ = W[q] / detJ;
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
            const double M11 = CC(0), M12 = CC(1), M13 = CC(2);
            const double M21 = !symmetric ? CC(3) : M12;
            const double M22 = !symmetric ? CC(4) : CC(3);
            const double M23 = !symmetric ? CC(5) : CC(4);
            const double M31 = !symmetric ? CC(6) : M13;
            const double M32 = !symmetric ? CC(7) : M23;
            const double M33 = !symmetric ? CC(8) : CC(5);
            const double R11 = M11 * A11 + M12 * A12 + M13 * A13;
            const double R12 = M11 * A21 + M12 * A22 + M13 * A23;
            const double R13 = M11 * A31 + M12 * A32 + M13 * A33;
            const double R21 = M21 * A11 + M22 * A12 + M23 * A13;
            const double R22 = M21 * A21 + M22 * A22 + M23 * A23;
            const double R23 = M21 * A31 + M22 * A32 + M23 * A33;
            const double R31 = M31 * A11 + M32 * A12 + M33 * A13;
            const double R32 = M31 * A21 + M32 * A22 + M33 * A23;
            const double R33 = M31 * A31 + M32 * A32 + M33 * A33;
            DD(0) = w_detJ * (A11 * R11 + A12 * R21 + A13 * R31);
            DD(1) = w_detJ * (A11 * R12 + A12 * R22 + A13 * R32);
            DD(2) = w_detJ * (A11 * R13 + A12 * R23 + A13 * R33);
            const double D22 = w_detJ * (A21 * R12 + A22 * R22 + A23 * R32);
            const double D23 = w_detJ * (A21 * R13 + A22 * R23 + A23 * R33);
            const double D33 = w_detJ * (A31 * R13 + A32 * R23 + A33 * R33);
            DD(4) = symmetric ? D23 : D22;
            DD(5) = symmetric ? D33 : D23;
            if (symmetric) { DD(3) = D22; }
            else
            {
               DD(3) = w_detJ * (A21 * R11 + A22 * R21 + A23 * R31);
               DD(6) = w_detJ * (A31 * R11 + A32 * R21 + A33 * R31);
               DD(7) = w_detJ * (A31 * R12 + A32 * R22 + A33 * R32);
               DD(8) = D33;
            }
         }
         else
         {
            const double C1 = CC(0);
            const double C2 = CC(coeff_dim == 3 ? 1 : 0);
            const double C3 = CC(coeff_dim == 3 ? 2 : 0);
            DD(0) = w_detJ * (C1 * A11 * A11 + C2 * A12 * A12 + C3 * A13 * A13);
            DD(1) = w_detJ * (C1 * A11 * A21 + C2 * A12 * A22 + C3 * A13 * A23);
            DD(2) = w_detJ * (C1 * A11 * A31 + C2 * A12 * A32 + C3 * A13 * A33);
            DD(3) = w_detJ * (C1 * A21 * A21 + C2 * A22 * A22 + C3 * A23 * A23);
            DD(4) = w_detJ * (C1 * A21 * A31 + C2 * A22 * A32 + C3 * A23 * A33);
            DD(5) = w_detJ * (C1 * A31 * A31 + C2 * A32 * A32 + C3 * A33 * A33);
         }
#undef JJ
#undef CC
#undef DD
      }
}

/* The body is inlined into size-specialised wrappers below: with D and Q
 * literal constants the compiler unrolls the contractions, as the
 * reference's compile-time kernel instances do on the CPU
 * (fem/integ/bilininteg_diffusion_kernels.cpp:64-83). The arithmetic and its
 * order are the same for every instance. */
static inline __attribute__((always_inline)) void
diff_apply_body(int ne, int symm, int d1d, int q1d, const double *B, const double *G,
                const double *Dq, const double *X, double *Y)
{
   const int D = d1d, Q = q1d, Q3 = Q * Q * Q, D3 = D * D * D, S = symm ? 6 : 9;
#pragma omp parallel for schedule(static)
   for (int e = 0; e < ne; ++e)
   {
      double grad[OR_MAXQ][OR_MAXQ][OR_MAXQ][3];
      const double *x = X + (long)D3 * e;
      double *y = Y + (long)D3 * e;
      const double *dq = Dq + (long)Q3 * S * e;
      for (int qz = 0; qz < Q; ++qz)
         for (int qy = 0; qy < Q; ++qy)
            for (int qx = 0; qx < Q; ++qx)
               grad[qz][qy][qx][0] = grad[qz][qy][qx][1] = grad[qz][qy][qx][2] = 0.0;
      for (int dz = 0; dz < D; ++dz)
      {
         double gXY[OR_MAXQ][OR_MAXQ][3];
         for (int qy = 0; qy < Q; ++qy)
            for (int qx = 0; qx < Q; ++qx)
               gXY[qy][qx][0] = gXY[qy][qx][1] = gXY[qy][qx][2] = 0.0;
         for (int dy = 0; dy < D; ++dy)
         {
            double gX[OR_MAXQ][2];
            for (int qx = 0; qx < Q; ++qx) { gX[qx][0] = gX[qx][1] = 0.0; }
            for (int dx = 0; dx < D; ++dx)
            {
               const double s = x[dx + D * (dy + D * dz)];
               for (int qx = 0; qx < Q; ++qx)
               {
                  gX[qx][0] += s * B[qx + Q * dx];
                  gX[qx][1] += s * G[qx + Q * dx];
               }
            }
            for (int qy = 0; qy < Q; ++qy)
            {
               const double wy = B[qy + Q * dy], wDy = G[qy + Q * dy];
               for (int qx = 0; qx < Q; ++qx)
               {
                  gXY[qy][qx][0] += gX[qx][1] * wy;
                  gXY[qy][qx][1] += gX[qx][0] * wDy;
                  gXY[qy][qx][2] += gX[qx][0] * wy;
               }
            }
         }
         for (int qz = 0; qz < Q; ++qz)
         {
            const double wz = B[qz + Q * dz], wDz = G[qz + Q * dz];
            for (int qy = 0; qy < Q; ++qy)
               for (int qx = 0; qx < Q; ++qx)
               {
                  grad[qz][qy][qx][0] += gXY[qy][qx][0] * wz;
                  grad[qz][qy][qx][1] += gXY[qy][qx][1] * wz;
                  grad[qz][qy][qx][2] += gXY[qy][qx][2] * wDz;
               }
         }
      }
      for (int qz = 0; qz < Q; ++qz)
         for (int qy = 0; qy < Q; ++qy)
            for (int qx = 0; qx < Q; ++qx)
            {
               const int q = qx + Q * (qy + Q * qz);
               const double O11 = dq[q], O12 = dq[q + Q3], O13 = dq[q + 2 * Q3];
               const double O21 = symm ? O12 : dq[q + 3 * Q3];
               const double O22 = symm ? dq[q + 3 * Q3] : dq[q + 4 * Q3];
               const double O23 = symm ? dq[q + 4 * Q3] : dq[q + 5 * Q3];
               const double O31 = symm ? O13 : dq[q + 6 * Q3];
               const double O32 = symm ? O23 : dq[q + 7 * Q3];
               const double O33 = symm ? dq[q + 5 * Q3] : dq[q + 8 * Q3];
               const double g0 = grad[qz][qy][qx][0], g1 = grad[qz][qy][qx][1],
                            g2 = grad[qz][qy][qx][2];
               grad[qz][qy][qx][0] = (O11 * g0) + (O12 * g1) + (O13 * g2);
               grad[qz][qy][qx][1] = (O21 * g0) + (O22 * g1) + (O23 * g2);
               grad[qz][qy][qx][2] = (O31 * g0) + (O32 * g1) + (O33 * g2);
            }
      for (int qz = 0; qz < Q; ++qz)
      {
         double gXY[OR_MAXQ][OR_MAXQ][3];
         for (int dy = 0; dy < D; ++dy)
            for (int dx = 0; dx < D; ++dx)
               gXY[dy][dx][0] = gXY[dy][dx][1] = gXY[dy][dx][2] = 0.0;
         for (int qy = 0; qy < Q; ++qy)
         {
            double gX[OR_MAXQ][3];
            for (int dx = 0; dx < D; ++dx) { gX[dx][0] = gX[dx][1] = gX[dx][2] = 0.0; }
            for (int qx = 0; qx < Q; ++qx)
            {
               const double g0 = grad[qz][qy][qx][0], g1 = grad[qz][qy][qx][1],
                            g2 = grad[qz][qy][qx][2];
               for (int dx = 0; dx < D; ++dx)
               {
                  const double wx = B[qx + Q * dx], wDx = G[qx + Q * dx];
                  gX[dx][0] += g0 * wDx;
                  gX[dx][1] += g1 * wx;
                  gX[dx][2] += g2 * wx;
               }
            }
            for (int dy = 0; dy < D; ++dy)
            {
               const double wy = B[qy + Q * dy], wDy = G[qy + Q * dy];
               for (int dx = 0; dx < D; ++dx)
               {
                  gXY[dy][dx][0] += gX[dx][0] * wy;
                  gXY[dy][dx][1] += gX[dx][1] * wDy;
                  gXY[dy][dx][2] += gX[dx][2] * wy;
               }
            }
         }
         for (int dz = 0; dz < D; ++dz)
         {
            const double wz = B[qz + Q * dz], wDz = G[qz + Q * dz];
            for (int dy = 0; dy < D; ++dy)
               for (int dx = 0; dx < D; ++dx)
                  y[dx + D * (dy + D * dz)] += (gXY[dy][dx][0] * wz) +
                                               (gXY[dy][dx][1] * wz) +
                                               (gXY[dy][dx][2] * wDz);
         }
      }
   }
}


#define OR_DIFF_CASE(d, q) \
   if (d1d == d && q1d == q) { diff_apply_body(ne, symm, d, q, B, G, Dq, X, Y); return; }

void or_diffusion_apply3d(int ne, int symm, int d1d, int q1d, const double *B,
                          const double *G, const double *Dq, const double *X,
                          double *Y)
{
   OR_DIFF_CASE(2, 3) OR_DIFF_CASE(3, 4) OR_DIFF_CASE(4, 5) OR_DIFF_CASE(5, 6)
   OR_DIFF_CASE(6, 7) OR_DIFF_CASE(7, 8) OR_DIFF_CASE(8, 9) OR_DIFF_CASE(9, 10)
   diff_apply_body(ne, symm, d1d, q1d, B, G, Dq, X, Y);
}
#undef OR_DIFF_CASE
void or_diffusion_diagonal3d(int ne, int symm, int d1d, int q1d,
                             const double *B, const double *G, const double *Dq,
                             double *Y)
{
   const int D = d1d, Q = q1d, Q3 = Q * Q * Q, D3 = D * D * D, S = symm ? 6 : 9;
#pragma omp parallel for schedule(static)
   for (int e = 0; e < ne; ++e)
   {
      double QQD[OR_MAXQ][OR_MAXQ][OR_MAXQ], QDD[OR_MAXQ][OR_MAXQ][OR_MAXQ];
      const double *dq = Dq + (long)Q3 * S * e;
      double *y = Y + (long)D3 * e;
      for (int i = 0; i < 3; ++i)
         for (int j = 0; j < 3; ++j)
         {
            const int ksym = j >= i ? 3 - (3 - i) * (2 - i) / 2 + j
                                    : 3 - (3 - j) * (2 - j) / 2 + i;
            const int k = symm ? ksym : i * 3 + j;
            for (int qx = 0; qx < Q; ++qx)
               for (int qy = 0; qy < Q; ++qy)
                  for (int dz = 0; dz < D; ++dz)
                  {
                     double s = 0.0;
                     for (int qz = 0; qz < Q; ++qz)
                     {
                        const int q = qx + (qy + qz * Q) * Q;
                        const double O = dq[q + Q3 * k];
                        const double Bz = B[qz + Q * dz], Gz = G[qz + Q * dz];
                        const double L = i == 2 ? Gz : Bz, R = j == 2 ? Gz : Bz;
                        s += L * O * R;
                     }
                     QQD[qx][qy][dz] = s;
                  }
            for (int qx = 0; qx < Q; ++qx)
               for (int dz = 0; dz < D; ++dz)
                  for (int dy = 0; dy < D; ++dy)
                  {
                     double s = 0.0;
                     for (int qy = 0; qy < Q; ++qy)
                     {
                        const double By = B[qy + Q * dy], Gy = G[qy + Q * dy];
                        const double L = i == 1 ? Gy : By, R = j == 1 ? Gy : By;
                        s += L * QQD[qx][qy][dz] * R;
                     }
                     QDD[qx][dy][dz] = s;
                  }
            for (int dz = 0; dz < D; ++dz)
               for (int dy = 0; dy < D; ++dy)
                  for (int dx = 0; dx < D; ++dx)
                  {
                     double s = y[dx + D * (dy + D * dz)];
                     for (int qx = 0; qx < Q; ++qx)
                     {
                        const double Bx = B[qx + Q * dx], Gx = G[qx + Q * dx];
                        const double L = i == 0 ? Gx : Bx, R = j == 0 ? Gx : Bx;
                        s += L * QDD[qx][dy][dz] * R;
                     }
                     y[dx + D * (dy + D * dz)] = s;
                  }
         }
   }
}

/* ---------------------------------------------------------------- mass */
void or_mass_setup3d(int ne, int nq, const double *W, const double *detJ,
                     const double *C, long c_size, int by_val, double *Dq)
{
   const int const_c = c_size == 1;
#pragma omp parallel for schedule(static)
   for (int e = 0; e < ne; ++e)
      for (int q = 0; q < nq; ++q)
      {
         const double dj = detJ[q + (long)nq * e];
         const double c = const_c ? C[0] : C[q + (long)nq * e];
         Dq[q + (long)nq * e] = W[q] * c * (by_val ? dj : 1.0 / dj);
      }
}

void or_mass_apply3d(int ne, int d1d, int q1d, const double *B,
                     const double *Dq, const double *X, double *Y)
{
   const int D = d1d, Q = q1d, Q3 = Q * Q * Q, D3 = D * D * D;
#pragma omp parallel for schedule(static)
   for (int e = 0; e < ne; ++e)
   {
      double sol[OR_MAXQ][OR_MAXQ][OR_MAXQ];
      const double *x = X + (long)D3 * e;
      double *y = Y + (long)D3 * e;
      const double *dq = Dq + (long)Q3 * e;
      for (int qz = 0; qz < Q; ++qz)
         for (int qy = 0; qy < Q; ++qy)
            for (int qx = 0; qx < Q; ++qx) { sol[qz][qy][qx] = 0.0; }
      for (int dz = 0; dz < D; ++dz)
      {
         double sxy[OR_MAXQ][OR_MAXQ];
         for (int qy = 0; qy < Q; ++qy)
            for (int qx = 0; qx < Q; ++qx) { sxy[qy][qx] = 0.0; }
         for (int dy = 0; dy < D; ++dy)
         {
            double sx[OR_MAXQ];
            for (int qx = 0; qx < Q; ++qx) { sx[qx] = 0.0; }
            for (int dx = 0; dx < D; ++dx)
            {
               const double s = x[dx + D * (dy + D * dz)];
               for (int qx = 0; qx < Q; ++qx) { sx[qx] += B[qx + Q * dx] * s; }
            }
            for (int qy = 0; qy < Q; ++qy)
            {
               const double wy = B[qy + Q * dy];
               for (int qx = 0; qx < Q; ++qx) { sxy[qy][qx] += wy * sx[qx]; }
            }
         }
         for (int qz = 0; qz < Q; ++qz)
         {
            const double wz = B[qz + Q * dz];
            for (int qy = 0; qy < Q; ++qy)
               for (int qx = 0; qx < Q; ++qx) { sol[qz][qy][qx] += wz * sxy[qy][qx]; }
         }
      }
      for (int qz = 0; qz < Q; ++qz)
         for (int qy = 0; qy < Q; ++qy)
            for (int qx = 0; qx < Q; ++qx)
               sol[qz][qy][qx] *= dq[qx + Q * (qy + Q * qz)];
      for (int qz = 0; qz < Q; ++qz)
      {
         double sxy[OR_MAXQ][OR_MAXQ];
         for (int dy = 0; dy < D; ++dy)
            for (int dx = 0; dx < D; ++dx) { sxy[dy][dx] = 0.0; }
         for (int qy = 0; qy < Q; ++qy)
         {
            double sx[OR_MAXQ];
            for (int dx = 0; dx < D; ++dx) { sx[dx] = 0.0; }
            for (int qx = 0; qx < Q; ++qx)
            {
               const double s = sol[qz][qy][qx];
               for (int dx = 0; dx < D; ++dx) { sx[dx] += B[qx + Q * dx] * s; }
            }
            for (int dy = 0; dy < D; ++dy)
            {
               const double wy = B[qy + Q * dy];
               for (int dx = 0; dx < D; ++dx) { sxy[dy][dx] += wy * sx[dx]; }
            }
         }
         for (int dz = 0; dz < D; ++dz)
         {
            const double wz = B[qz + Q * dz];
            for (int dy = 0; dy < D; ++dy)
               for (int dx = 0; dx < D; ++dx)
                  y[dx + D * (dy + D * dz)] += wz * sxy[dy][dx];
         }
      }
   }
}

void or_mass_diagonal3d(int ne, int d1d, int q1d, const double *B,
                        const double *Dq, double *Y)
{
   const int D = d1d, Q = q1d, Q3 = Q * Q * Q, D3 = D * D * D;
#pragma omp parallel for schedule(static)
   for (int e = 0; e < ne; ++e)
   {
      double QQD[OR_MAXQ][OR_MAXQ][OR_MAXQ], QDD[OR_MAXQ][OR_MAXQ][OR_MAXQ];
      const double *dq = Dq + (long)Q3 * e;
      double *y = Y + (long)D3 * e;
      for (int qx = 0; qx < Q; ++qx)
         for (int qy = 0; qy < Q; ++qy)
            for (int dz = 0; dz < D; ++dz)
            {
               double s = 0.0;
               for (int qz = 0; qz < Q; ++qz)
                  s += B[qz + Q * dz] * B[qz + Q * dz] * dq[qx + Q * (qy + Q * qz)];
               QQD[qx][qy][dz] = s;
            }
      for (int qx = 0; qx < Q; ++qx)
         for (int dz = 0; dz < D; ++dz)
            for (int dy = 0; dy < D; ++dy)
            {
               double s = 0.0;
               for (int qy = 0; qy < Q; ++qy)
                  s += B[qy + Q * dy] * B[qy + Q * dy] * QQD[qx][qy][dz];
               QDD[qx][dy][dz] = s;
            }
      for (int dz = 0; dz < D; ++dz)
         for (int dy = 0; dy < D; ++dy)
            for (int dx = 0; dx < D; ++dx)
            {
               double t = 0.0;
               for (int qx = 0; qx < Q; ++qx)
                  t += B[qx + Q * dx] * B[qx + Q * dx] * QDD[qx][dy][dz];
               y[dx + D * (dy + D * dz)] += t;
            }
   }
}

/* ------------------------------------------------------- L-vector apply */
void or_pa_mult(int kind, int ne, int ndofs, int symm, int d1d, int q1d,
                const int *gather_map, const int *offsets, const int *indices,
                const double *B, const double *G, const double *Dq,
                const double *x, double *y, double *work)
{
   const long nE = (long)ne * d1d * d1d * d1d;
   double *xE = work, *yE = work + nE;
   or_restriction_mult(ne, d1d * d1d * d1d, gather_map, x, xE);
   memset(yE, 0, sizeof(double) * nE);
   if (kind == 0) { or_diffusion_apply3d(ne, symm, d1d, q1d, B, G, Dq, xE, yE); }
   else { or_mass_apply3d(ne, d1d, q1d, B, Dq, xE, yE); }
   or_restriction_mult_transpose(d1d * d1d * d1d, ndofs, offsets, indices, yE, y, 0);
}

/* fem/bilinearform_ext.cpp:807-847: the integrator's apply into a zeroed
 * temporary E-vector, then AddWithMarkers_ (:753-774) adds the marked
 * elements' blocks to localY, which MultTranspose scatters (:548-556). */
void or_pa_mult_markers(int kind, int ne, int ndofs, int symm, int d1d, int q1d,
                        const int *gather_map, const int *offsets, const int *indices,
                        const double *B, const double *G, const double *Dq,
                        const int *attributes, const int *markers,
                        const double *x, double *y, double *work)
{
   const int nd = d1d * d1d * d1d;
   const long nE = (long)ne * nd;
   double *xE = work, *tE = work + nE, *yE = work + 2 * nE;
   or_restriction_mult(ne, nd, gather_map, x, xE);
   memset(tE, 0, sizeof(double) * nE);
   memset(yE, 0, sizeof(double) * nE);
   if (kind == 0) { or_diffusion_apply3d(ne, symm, d1d, q1d, B, G, Dq, xE, tE); }
   else { or_mass_apply3d(ne, d1d, q1d, B, Dq, xE, tE); }
   for (int e = 0; e < ne; ++e)
   {
      const int a = attributes[e];
      if (a <= 0 || markers[a - 1] == 0) { continue; }
      for (int i = 0; i < nd; ++i) { yE[(long)e * nd + i] += tE[(long)e * nd + i]; }
   }
   or_restriction_mult_transpose(nd, ndofs, offsets, indices, yE, y, 0);
}

/* ----------------------------------------------------------------- PCG */
static double dot(int n, const double *a, const double *b)
{
   double s = 0.0;
   for (int i = 0; i < n; ++i) { s += a[i] * b[i]; }
   return s;
}

typedef struct
{
   int ne, ndofs, symm, d1d, q1d;
   const int *gm, *off, *ind;
   const double *B, *G, *D;
   const int *ess; int n_ess;
   double *work, *z;
} or_cop;

/* ConstrainedOperator::Mult, DIAG_ONE (linalg/operator.cpp:601-661) */
static void cop_mult(const or_cop *A, const double *x, double *y)
{
   memcpy(A->z, x, sizeof(double) * A->ndofs);
   for (int i = 0; i < A->n_ess; ++i) { A->z[A->ess[i]] = 0.0; }
   or_pa_mult(0, A->ne, A->ndofs, A->symm, A->d1d, A->q1d, A->gm, A->off,
              A->ind, A->B, A->G, A->D, A->z, y, A->work);
   for (int i = 0; i < A->n_ess; ++i) { y[A->ess[i]] = x[A->ess[i]]; }
}

int or_pcg_diffusion(int ne, int ndofs, int symm, int d1d, int q1d,
                     const int *gather_map, const int *offsets,
                     const int *indices, const double *B, const double *G,
                     const double *Dq, const int *ess, int n_ess,
                     const double *dinv, const double *b, double *x,
                     double rel_tol, double abs_tol, int max_it,
                     int iterative_mode, double *final_norm, int *converged)
{
   const int n = ndofs;
   const long nE = (long)ne * d1d * d1d * d1d;
   double *r = (double *)malloc(sizeof(double) * n);
   double *d = (double *)malloc(sizeof(double) * n);
   double *z = (double *)malloc(sizeof(double) * n);
   double *zz = (double *)malloc(sizeof(double) * n);
   double *work = (double *)malloc(sizeof(double) * 2 * nE);
   or_cop A = {ne, ndofs, symm, d1d, q1d, gather_map, offsets, indices,
               B, G, Dq, ess, n_ess, work, zz};
   int i, final_iter = 0;
   double nom, nom0, den, betanom = 0.0, alpha, beta, r0;
   if (iterative_mode)
   {
      cop_mult(&A, x, r);
      for (int k = 0; k < n; ++k) { r[k] = b[k] - r[k]; }
   }
   else
   {
      memcpy(r, b, sizeof(double) * n);
      memset(x, 0, sizeof(double) * n);
   }
   /* OperatorJacobiSmoother::Mult, non-iterative mode: z = dinv .* r */
   for (int k = 0; k < n; ++k) { z[k] = dinv[k] * r[k]; d[k] = z[k]; }
   nom0 = nom = dot(n, d, r);
   *converged = 0;
   if (nom < 0.0 || !isfinite(nom)) { *final_norm = nom; goto done; }
   r0 = fmax(nom * rel_tol * rel_tol, abs_tol * abs_tol);
   if (nom <= r0) { *converged = 1; *final_norm = sqrt(nom); goto done; }
   cop_mult(&A, d, z);
   den = dot(n, z, d);
   if (den == 0.0) { *final_norm = sqrt(nom); goto done; }
   final_iter = max_it;
   for (i = 1; 1;)
   {
      alpha = nom / den;
      for (int k = 0; k < n; ++k) { x[k] += alpha * d[k]; }
      for (int k = 0; k < n; ++k) { r[k] += -alpha * z[k]; }
      for (int k = 0; k < n; ++k) { z[k] = dinv[k] * r[k]; }
      betanom = dot(n, r, z);
      if (betanom < 0.0 || !isfinite(betanom)) { final_iter = i; break; }
      if (betanom <= r0) { *converged = 1; final_iter = i; break; }
      if (++i > max_it) { break; }
      beta = betanom / nom;
      for (int k = 0; k < n; ++k) { d[k] = z[k] + beta * d[k]; }
      cop_mult(&A, d, z);
      den = dot(n, d, z);
      if (den == 0.0) { final_iter = i; break; }
      nom = betanom;
   }
   *final_norm = sqrt(betanom);
   (void)nom0;
done:
   free(r); free(d); free(z); free(zz); free(work);
   return final_iter;
}

/* ------------------------------------------------------------ p-multigrid */
/* CGSolver::Mult (linalg/solvers.cpp:869-1050) with a general
 * preconditioner (prec == NULL: plain CG, z = r), zero initial guess. */
typedef void (*or_prec_fn)(void *ctx, const double *r, double *z);
static int pcg_generic(const or_cop *A, or_prec_fn prec, void *pctx, const double *b,
                       double *x, double rel_tol, double abs_tol, int max_it,
                       double *final_norm, int *converged)
{
   const int n = A->ndofs;
   double *r = (double *)malloc(sizeof(double) * n);
   double *d = (double *)malloc(sizeof(double) * n);
   double *z = (double *)malloc(sizeof(double) * n);
   int i, final_iter = 0;
   double nom, den, betanom = 0.0, alpha, beta, r0;
   memcpy(r, b, sizeof(double) * n);
   memset(x, 0, sizeof(double) * n);
   if (prec) { prec(pctx, r, z); } else { memcpy(z, r, sizeof(double) * n); }
   memcpy(d, z, sizeof(double) * n);
   nom = dot(n, d, r);
   *converged = 0;
   if (nom < 0.0 || !isfinite(nom)) { *final_norm = nom; goto done; }
   r0 = fmax(nom * rel_tol * rel_tol, abs_tol * abs_tol);
   if (nom <= r0) { *converged = 1; *final_norm = sqrt(nom); goto done; }
   cop_mult(A, d, z);
   den = dot(n, z, d);
   if (den == 0.0) { *final_norm = sqrt(nom); goto done; }
   final_iter = max_it;
   for (i = 1; 1;)
   {
      alpha = nom / den;
      for (int k = 0; k < n; ++k) { x[k] += alpha * d[k]; }
      for (int k = 0; k < n; ++k) { r[k] += -alpha * z[k]; }
      if (prec) { prec(pctx, r, z); } else { memcpy(z, r, sizeof(double) * n); }
      betanom = dot(n, r, z);
      if (betanom < 0.0 || !isfinite(betanom)) { final_iter = i; break; }
      if (betanom <= r0) { *converged = 1; final_iter = i; break; }
      if (++i > max_it) { break; }
      beta = betanom / nom;
      for (int k = 0; k < n; ++k) { d[k] = z[k] + beta * d[k]; }
      cop_mult(A, d, z);
      den = dot(n, d, z);
      if (den == 0.0) { final_iter = i; break; }
      nom = betanom;
   }
   *final_norm = sqrt(betanom);
done:
   free(r); free(d); free(z);
   return final_iter;
}

/* ElementRestriction::BooleanMask (fem/restriction.cpp:255-292): 1 on the
 * first element slot of each dof's CSR row, 0 on its other slots. */
void or_boolean_mask(int ndofs, int nslots, const int *offsets, const int *indices,
                     double *mask)
{
   for (int s = 0; s < nslots; ++s) { mask[s] = 0.0; }
   for (int i = 0; i < ndofs; ++i)
   {
      if (offsets[i + 1] > offsets[i])
      {
         const int s = indices[offsets[i]];
         mask[s >= 0 ? s : -1 - s] = 1.0;
      }
   }
}

/* y(qx,qy,qz) = sum Bi(qx,dx) Bi(qy,dy) Bi(qz,dz) x(dx,dy,dz) per element
 * (Bi: (df, dc)); transpose != 0 applies the transposed contraction
 * (fem/transfer.cpp:2703-2934, TransferKernels::{Prolongation,Restriction}3D). */
static void interp3d(int ne, int dc, int df, const double *Bi, const double *x, double *y,
                     int transpose)
{
   const int n_in = transpose ? df : dc, n_out = transpose ? dc : df;
   const long in3 = (long)n_in * n_in * n_in, out3 = (long)n_out * n_out * n_out;
   double *t1 = (double *)malloc(sizeof(double) * n_out * n_in * n_in);
   double *t2 = (double *)malloc(sizeof(double) * n_out * n_out * n_in);
   for (int e = 0; e < ne; ++e)
   {
      const double *xe = x + e * in3;
      double *ye = y + e * out3;
      /* M(o, i) = Bi(o, i) (prolong) or Bi(i, o) (transpose) */
#define MI(o, i) (transpose ? Bi[(i) + df * (o)] : Bi[(o) + df * (i)])
      for (int k = 0; k < n_in; ++k)
         for (int j = 0; j < n_in; ++j)
            for (int o = 0; o < n_out; ++o)
            {
               double s = 0.0;
               for (int i = 0; i < n_in; ++i) { s += MI(o, i) * xe[i + n_in * (j + n_in * k)]; }
               t1[o + n_out * (j + n_in * k)] = s;
            }
      for (int k = 0; k < n_in; ++k)
         for (int o2 = 0; o2 < n_out; ++o2)
            for (int o = 0; o < n_out; ++o)
            {
               double s = 0.0;
               for (int j = 0; j < n_in; ++j) { s += MI(o2, j) * t1[o + n_out * (j + n_in * k)]; }
               t2[o + n_out * (o2 + n_out * k)] = s;
            }
      for (int o3 = 0; o3 < n_out; ++o3)
         for (int o2 = 0; o2 < n_out; ++o2)
            for (int o = 0; o < n_out; ++o)
            {
               double s = 0.0;
               for (int k = 0; k < n_in; ++k) { s += MI(o3, k) * t2[o + n_out * (o2 + n_out * k)]; }
               ye[o + n_out * (o2 + n_out * o3)] = s;
            }
#undef MI
   }
   free(t1); free(t2);
}

/* TensorProductPRefinementTransferOperator::Mult (fem/transfer.cpp:2939-2963):
 * y_f = R_f^T (mask .* I (R_c x_c)). */
void or_ptransfer_mult(const or_mg_level *c, const or_mg_level *f, const double *x, double *y)
{
   const int ne = c->ne, dc = c->d1d, df = f->d1d;
   const long nc = (long)ne * dc * dc * dc, nf = (long)ne * df * df * df;
   double *xe = (double *)malloc(sizeof(double) * nc);
   double *ye = (double *)malloc(sizeof(double) * nf);
   double *mask = (double *)malloc(sizeof(double) * nf);
   or_restriction_mult(ne, dc * dc * dc, c->gather_map, x, xe);
   interp3d(ne, dc, df, f->Bi, xe, ye, 0);
   or_boolean_mask(f->ndofs, (int)nf, f->offsets, f->indices, mask);
   for (long s = 0; s < nf; ++s) { ye[s] *= mask[s]; }
   or_restriction_mult_transpose(df * df * df, f->ndofs, f->offsets, f->indices, ye, y, 0);
   free(xe); free(ye); free(mask);
}

/* ::MultTranspose (fem/transfer.cpp:2965-2989): y_c = R_c^T I^T (mask .* R_f x_f). */
void or_ptransfer_mult_transpose(const or_mg_level *c, const or_mg_level *f, const double *x,
                                 double *y)
{
   const int ne = c->ne, dc = c->d1d, df = f->d1d;
   const long nc = (long)ne * dc * dc * dc, nf = (long)ne * df * df * df;
   double *xe = (double *)malloc(sizeof(double) * nf);
   double *ye = (double *)malloc(sizeof(double) * nc);
   double *mask = (double *)malloc(sizeof(double) * nf);
   or_restriction_mult(ne, df * df * df, f->gather_map, x, xe);
   or_boolean_mask(f->ndofs, (int)nf, f->offsets, f->indices, mask);
   for (long s = 0; s < nf; ++s) { xe[s] *= mask[s]; }
   interp3d(ne, dc, df, f->Bi, xe, ye, 1);
   or_restriction_mult_transpose(dc * dc * dc, c->ndofs, c->offsets, c->indices, ye, y, 0);
   free(xe); free(ye); free(mask);
}

/* Chebyshev smoother coefficients (linalg/solvers.cpp:552-616 states them
 * in closed form for orders 1-5): with the interval [0.3, 1.2] * lambda,
 * theta its centre and delta its half width, the smoother is
 * y = p(D^-1 A) D^-1 x where 1 - t p(t) = T_k((theta - t)/delta) /
 * T_k(theta/delta). Derived here by expanding the Chebyshev recurrence
 * T_{m+1} = 2 s T_m - T_{m-1} at s = (theta - t)/delta as polynomials in t:
 * c_{j-1} = -e_j / e_0 for T_k(s(t)) = sum_j e_j t^j. */
void or_chebyshev_coeffs(int order, double lambda, double *c)
{
   const double up = 1.2 * lambda, lo = 0.3 * lambda;
   const double theta = 0.5 * (up + lo), delta = 0.5 * (up - lo);
   const double a = theta / delta, b = -1.0 / delta;
   double Pm[16] = {0}, P[16] = {0}, Pn[16];
   Pm[0] = 1.0;                 /* T_0 */
   P[0] = a; P[1] = b;          /* T_1 */
   if (order == 1) { memcpy(Pm, P, sizeof(P)); }
   for (int m = 1; m < order; ++m)
   {
      for (int j = 0; j <= m + 1; ++j)
      {
         double v = 2.0 * a * P[j] - Pm[j];
         if (j > 0) { v += 2.0 * b * P[j - 1]; }
         Pn[j] = v;
      }
      for (int j = m + 2; j < 16; ++j) { Pn[j] = 0.0; }
      memcpy(Pm, P, sizeof(P));
      memcpy(P, Pn, sizeof(P));
   }
   const double *T = order == 1 ? Pm : P;
   for (int j = 1; j <= order; ++j) { c[j - 1] = -T[j] / T[0]; }
}

static void level_cop(const or_mg_level *l, or_cop *A, double *work, double *zz)
{
   or_cop t = {l->ne, l->ndofs, 1, l->d1d, l->q1d, l->gather_map, l->offsets, l->indices,
               l->B, l->G, l->qdata, l->ess, l->n_ess, work, zz};
   *A = t;
}
static double *level_dinv(const or_mg_level *l)
{
   double *dinv = (double *)malloc(sizeof(double) * l->ndofs);
   for (int i = 0; i < l->ndofs; ++i) { dinv[i] = 1.0 / l->diag[i]; }
   for (int i = 0; i < l->n_ess; ++i) { dinv[l->ess[i]] = 1.0; }
   return dinv;
}

/* OperatorChebyshevSmoother::Mult (linalg/solvers.cpp:619-656) */
void or_chebyshev_mult(const or_mg_level *l, int order, const double *x, double *y)
{
   const int n = l->ndofs;
   const long nE = (long)l->ne * l->d1d * l->d1d * l->d1d;
   double coeffs[16];
   or_chebyshev_coeffs(order, l->lambda, coeffs);
   double *dinv = level_dinv(l);
   double *res = (double *)malloc(sizeof(double) * n);
   double *h = (double *)malloc(sizeof(double) * n);
   double *work = (double *)malloc(sizeof(double) * 2 * nE);
   double *zz = (double *)malloc(sizeof(double) * n);
   or_cop A;
   level_cop(l, &A, work, zz);
   memcpy(res, x, sizeof(double) * n);
   for (int i = 0; i < n; ++i) { y[i] = 0.0; }
   for (int k = 0; k < order; ++k)
   {
      if (k > 0)
      {
         cop_mult(&A, res, h);
         memcpy(res, h, sizeof(double) * n);
      }
      for (int i = 0; i < n; ++i) { res[i] *= dinv[i]; }
      for (int i = 0; i < n; ++i) { y[i] += coeffs[k] * res[i]; }
   }
   free(dinv); free(res); free(h); free(work); free(zz);
}

/* splitmix64 at counter i: the i-th draw of the stream seeded with `seed`,
 * as a double in [0, 1) */
static double sm_u01(unsigned long long seed, long i)
{
   unsigned long long z = seed + (unsigned long long)(i + 1) * 0x9e3779b97f4a7c15ULL;
   z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
   z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
   z ^= z >> 31;
   return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

/* PowerMethod::EstimateLargestEigenvalue (linalg/operator.cpp:886-942) on
 * D^-1 A (OperatorJacobiSmoother with ess entries 1, linalg/solvers.cpp:
 * 493-510); the start vector is the splitmix64 stream of `seed`. */
double or_power_method(const or_mg_level *l, int steps, double tol, unsigned long long seed)
{
   const int n = l->ndofs;
   const long nE = (long)l->ne * l->d1d * l->d1d * l->d1d;
   double *dinv = level_dinv(l);
   double *v0 = (double *)malloc(sizeof(double) * n);
   double *v1 = (double *)malloc(sizeof(double) * n);
   double *work = (double *)malloc(sizeof(double) * 2 * nE);
   double *zz = (double *)malloc(sizeof(double) * n);
   or_cop A;
   level_cop(l, &A, work, zz);
   for (int i = 0; i < n; ++i) { v0[i] = sm_u01(seed, i); }
   double lam = 1.0;
   for (int it = 0; it < steps; ++it)
   {
      const double nrm = sqrt(dot(n, v0, v0));
      for (int i = 0; i < n; ++i) { v0[i] /= nrm; }
      cop_mult(&A, v0, v1);
      for (int i = 0; i < n; ++i) { v1[i] *= dinv[i]; }
      const double ln = dot(n, v0, v1);
      const double diff = fabs((ln - lam) / lam);
      lam = ln;
      double *t = v0; v0 = v1; v1 = t;
      if (diff < tol) { break; }
   }
   free(dinv); free(v0); free(v1); free(work); free(zz);
   return lam;
}

typedef struct
{
   const or_mg_level *lv;
   int order;
   double coarse_tol;
   int coarse_max;
} or_mg;

/* MultigridBase::Cycle, V-cycle with one pre- and one post-smoothing step
 * (fem/multigrid.cpp:147-239): X = right-hand side, Y = correction. */
static void mg_cycle(const or_mg *M, int level, const double *X, double *Y)
{
   const or_mg_level *l = M->lv + level;
   const int n = l->ndofs;
   const long nE = (long)l->ne * l->d1d * l->d1d * l->d1d;
   double *work = (double *)malloc(sizeof(double) * 2 * nE);
   double *zz = (double *)malloc(sizeof(double) * n);
   or_cop A;
   level_cop(l, &A, work, zz);
   if (level == 0)
   {
      double fn; int conv;
      pcg_generic(&A, NULL, NULL, X, Y, M->coarse_tol, 0.0, M->coarse_max, &fn, &conv);
      free(work); free(zz);
      return;
   }
   const or_mg_level *c = M->lv + level - 1;
   double *R = (double *)malloc(sizeof(double) * n);
   double *Z = (double *)malloc(sizeof(double) * n);
   double *Xc = (double *)malloc(sizeof(double) * c->ndofs);
   double *Yc = (double *)malloc(sizeof(double) * c->ndofs);
   or_chebyshev_mult(l, M->order, X, Y);                  /* pre-smooth, zero guess */
   cop_mult(&A, Y, R);
   for (int i = 0; i < n; ++i) { R[i] = X[i] - R[i]; }
   or_ptransfer_mult_transpose(c, l, R, Xc);
   for (int i = 0; i < c->ndofs; ++i) { Yc[i] = 0.0; }
   mg_cycle(M, level - 1, Xc, Yc);
   or_ptransfer_mult(c, l, Yc, Z);
   for (int i = 0; i < n; ++i) { Y[i] += Z[i]; }
   cop_mult(&A, Y, R);                                    /* post-smooth */
   for (int i = 0; i < n; ++i) { R[i] = X[i] - R[i]; }
   or_chebyshev_mult(l, M->order, R, Z);
   for (int i = 0; i < n; ++i) { Y[i] += Z[i]; }
   free(R); free(Z); free(Xc); free(Yc); free(work); free(zz);
}

void or_mg_mult(const or_mg_level *lv, int nl, int order, double coarse_tol, int coarse_max,
                const double *x, double *y)
{
   or_mg M = {lv, order, coarse_tol, coarse_max};
   for (int i = 0; i < lv[nl - 1].ndofs; ++i) { y[i] = 0.0; }
   mg_cycle(&M, nl - 1, x, y);
}

typedef struct { or_mg M; int nl; } or_mg_ctx;
static void mg_prec_top(void *ctx, const double *r, double *z)
{
   const or_mg_ctx *C = (const or_mg_ctx *)ctx;
   for (int i = 0; i < C->M.lv[C->nl - 1].ndofs; ++i) { z[i] = 0.0; }
   mg_cycle(&C->M, C->nl - 1, r, z);
}

/* CGSolver::Mult preconditioned by the V-cycle (the fine level's
 * constrained operator); returns the iteration count. */
int or_mg_pcg(const or_mg_level *lv, int nl, int order, double coarse_tol, int coarse_max,
              const double *b, double *x, double rel_tol, double abs_tol, int max_it,
              double *final_norm, int *converged)
{
   const or_mg_level *f = lv + nl - 1;
   const long nE = (long)f->ne * f->d1d * f->d1d * f->d1d;
   double *work = (double *)malloc(sizeof(double) * 2 * nE);
   double *zz = (double *)malloc(sizeof(double) * f->ndofs);
   or_cop A;
   level_cop(f, &A, work, zz);
   or_mg_ctx C = {{lv, order, coarse_tol, coarse_max}, nl};
   const int it = pcg_generic(&A, mg_prec_top, &C, b, x, rel_tol, abs_tol, max_it, final_norm,
                              converged);
   free(work); free(zz);
   return it;
}

/* ------------------------------------------------------------ linear form */
/* DomainLFIntegrator::AssembleDevice + LinearFormExtension::Assemble
 * (fem/integ/lininteg_domain.cpp:22-59, DLFEvalAssemble3D in
 * fem/integ/lininteg_domain_kernels.hpp:164-..., fem/linearform_ext.cpp:20-68):
 * y_e(dx,dy,dz) = sum_q B(qx,dx) B(qy,dy) B(qz,dz) W(q) f(q,e) detJ(q,e),
 * b = R^T y. f has c_size 1 (constant) or Q^3 NE values. */
void or_domain_lf3d(int ne, int d1d, int q1d, const double *B, const double *W,
                    const double *detJ, const double *f, long c_size, int ndofs,
                    const int *offsets, const int *indices, double *b)
{
   const int D = d1d, Q = q1d, D3 = D * D * D, Q3 = Q * Q * Q;
   double *yE = (double *)malloc(sizeof(double) * (size_t)ne * D3);
#pragma omp parallel for
   for (int e = 0; e < ne; ++e)
   {
      double *t1 = (double *)malloc(sizeof(double) * D * Q * Q);
      double *t2 = (double *)malloc(sizeof(double) * D * D * Q);
      double v[4096];
      for (int q = 0; q < Q3; ++q)
      {
         const double fv = c_size == 1 ? f[0] : f[q + (long)Q3 * e];
         v[q] = W[q] * fv * detJ[q + (long)Q3 * e];
      }
      /* contract x, then y, then z */
      for (int qz = 0; qz < Q; ++qz)
         for (int qy = 0; qy < Q; ++qy)
            for (int dx = 0; dx < D; ++dx)
            {
               double s = 0.0;
               for (int qx = 0; qx < Q; ++qx) { s += B[qx + Q * dx] * v[qx + Q * (qy + Q * qz)]; }
               t1[dx + D * (qy + Q * qz)] = s;
            }
      for (int qz = 0; qz < Q; ++qz)
         for (int dy = 0; dy < D; ++dy)
            for (int dx = 0; dx < D; ++dx)
            {
               double s = 0.0;
               for (int qy = 0; qy < Q; ++qy) { s += B[qy + Q * dy] * t1[dx + D * (qy + Q * qz)]; }
               t2[dx + D * (dy + D * qz)] = s;
            }
      for (int dz = 0; dz < D; ++dz)
         for (int dy = 0; dy < D; ++dy)
            for (int dx = 0; dx < D; ++dx)
            {
               double s = 0.0;
               for (int qz = 0; qz < Q; ++qz) { s += B[qz + Q * dz] * t2[dx + D * (dy + D * qz)]; }
               yE[(long)e * D3 + dx + D * (dy + D * dz)] = s;
            }
      free(t1); free(t2);
   }
   or_restriction_mult_transpose(D3, ndofs, offsets, indices, yE, b, 0);
   free(yE);
}
