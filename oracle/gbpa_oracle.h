/* CPU oracle for the partial-assembly H1 path: a plain-C restatement of the
 * reference's algorithms, used ONLY as the checker by tests/, by smoke() and by
 * bench.py's CPU-baseline leg. It is never linked into or called by the GPU
 * library. Every function cites the reference file:line it restates.
 *
 * Layouts are the reference's column-major ones:
 *   B, G        (Q, D)            B[q + Q*d]
 *   W           (Q, Q, Q)
 *   J           (Q, Q, Q, 3, 3, NE)  J[q + Q3*(row + 3*(col + 3*e))]
 *   qdata diff  (Q, Q, Q, S, NE)  S = 6 (symmetric) or 9
 *   qdata mass  (Q, Q, Q, NE)
 *   E-vector    (D, D, D, NE)
 */
#ifndef GBPA_ORACLE_H
#define GBPA_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* fem/restriction.cpp:26-114 (vdim = 1) */
void or_restriction_build(int ne, int dof, int ndofs, const int *elem_dofs,
                          const int *dof_map, int *offsets, int *indices,
                          int *gather_map);
/* fem/restriction.cpp:116-136 */
void or_restriction_mult(int ne, int nd, const int *gather_map,
                         const double *x, double *y);
/* fem/restriction.cpp:159-201; add != 0 accumulates into y */
void or_restriction_mult_transpose(int nd, int ndofs, const int *offsets,
                                   const int *indices, const double *x,
                                   double *y, int add);
/* fem/restriction.cpp:203-228 */
void or_restriction_abs_mult_transpose(int nd, int ndofs, const int *offsets,
                                       const int *indices, const double *x,
                                       double *y);

/* fem/intrules.cpp:620-690 (Gauss-Legendre on [0,1]) */
void or_gauss_legendre(int n, double *x, double *w);
/* fem/intrules.cpp:708-800 (Gauss-Lobatto points on [0,1]) */
void or_gauss_lobatto(int n, double *x);
/* fem/fe/fe_base.cpp:2697-2741: B[q + Q*d] = phi_d(xq), G = phi_d'(xq) for
 * the Lagrange basis on the np = D nodes `nodes` at the Q points `xq`. */
void or_basis_tables(int D, const double *nodes, int Q, const double *xq,
                     double *B, double *G);

/* fem/qinterp/grad.hpp:233-376 (byNODES, reference-space derivatives):
 * J(q, c, d, e) = d x_c / d xi_d from the lexicographic nodes E-vector
 * X (Dg, Dg, Dg, 3, NE). */
void or_geom_jacobians3d(int ne, int dg, int q1d, const double *Bg,
                         const double *Gg, const double *X, double *J);
/* determinant of each J (fem/qinterp/det.hpp:253-330) */
void or_geom_det3d(int ne, const double *J, int q3, double *detJ);

/* fem/integ/bilininteg_diffusion_kernels.cpp:262-386. c_size = coeff_dim
 * (constant) or coeff_dim*Q^3*NE. */
void or_diffusion_setup3d(int ne, int q1d, int coeff_dim, const double *W,
                          const double *J, const double *C, long c_size,
                          double *D);
/* fem/integ/bilininteg_diffusion_kernels.hpp:796-986 (accumulates y) */
void or_diffusion_apply3d(int ne, int symm, int d1d, int q1d, const double *B,
                          const double *G, const double *D, const double *x,
                          double *y);
/* fem/integ/bilininteg_diffusion_kernels.hpp:268-366 (accumulates y) */
void or_diffusion_diagonal3d(int ne, int symm, int d1d, int q1d,
                             const double *B, const double *G, const double *D,
                             double *y);
/* fem/integ/bilininteg_mass_pa.cpp:73-89: v = W * c * detJ (by_val) or W*c/detJ */
void or_mass_setup3d(int ne, int nq, const double *W, const double *detJ,
                     const double *C, long c_size, int by_val, double *D);
/* fem/integ/bilininteg_mass_kernels.hpp:664-813 (accumulates y) */
void or_mass_apply3d(int ne, int d1d, int q1d, const double *B,
                     const double *D, const double *x, double *y);
/* fem/integ/bilininteg_mass_kernels.hpp:262-329 (accumulates y) */
void or_mass_diagonal3d(int ne, int d1d, int q1d, const double *B,
                        const double *D, double *y);

/* PABilinearFormExtension::MultInternal, fem/bilinearform_ext.cpp:487-564:
 * y = R^T A_e R x for one integrator; kind 0 = diffusion, 1 = mass.
 * work: 2*ne*D^3 doubles. */
void or_pa_mult(int kind, int ne, int ndofs, int symm, int d1d, int q1d,
                const int *gather_map, const int *offsets, const int *indices,
                const double *B, const double *G, const double *D,
                const double *x, double *y, double *work);

/* PABilinearFormExtension::AddMultWithMarkers, fem/bilinearform_ext.cpp:
 * 530-550 and 807-847: y = R^T sum_e [marked e] A_e R x, where element e is
 * marked iff attributes[e] > 0 and markers[attributes[e] - 1] != 0
 * (AddWithMarkers_, :753-774). kind 0 = diffusion, 1 = mass. work: 3*ne*D^3
 * doubles. */
void or_pa_mult_markers(int kind, int ne, int ndofs, int symm, int d1d, int q1d,
                        const int *gather_map, const int *offsets, const int *indices,
                        const double *B, const double *G, const double *D,
                        const int *attributes, const int *markers,
                        const double *x, double *y, double *work);

/* CGSolver::Mult (linalg/solvers.cpp:869-1050) with OperatorJacobiSmoother
 * (linalg/solvers.cpp:401-452) on ConstrainedOperator (linalg/operator.cpp:
 * 601-661, DIAG_ONE) around the PA diffusion operator. dinv is the smoother's
 * inverse diagonal (ess entries already set to 1). Returns iterations;
 * *final_norm = sqrt(betanom); *converged set. x is the initial guess when
 * iterative_mode != 0 and is overwritten with the solution. */
int or_pcg_diffusion(int ne, int ndofs, int symm, int d1d, int q1d,
                     const int *gather_map, const int *offsets,
                     const int *indices, const double *B, const double *G,
                     const double *D, const int *ess, int n_ess,
                     const double *dinv, const double *b, double *x,
                     double rel_tol, double abs_tol, int max_it,
                     int iterative_mode, double *final_norm, int *converged);

/* ---- p-multigrid (examples/ex26.cpp structure). One level of the
 * hierarchy: its symmetric PA diffusion operator (constrained by ess), the
 * unconstrained diagonal and eigenvalue estimate of D^-1 A for its
 * Chebyshev smoother, and Bi (d1d, d1d of the level below): the coarser
 * level's Lagrange basis at this level's lexicographic nodes. */
typedef struct or_mg_level
{
   int ne, ndofs, d1d, q1d;
   const int *gather_map, *offsets, *indices;
   const double *B, *G, *qdata;
   const int *ess;
   int n_ess;
   const double *diag;
   double lambda;
   const double *Bi;
} or_mg_level;

/* fem/restriction.cpp:255-292 */
void or_boolean_mask(int ndofs, int nslots, const int *offsets, const int *indices,
                     double *mask);
/* fem/transfer.cpp:2939-2989 (c: coarse level, f: fine level) */
void or_ptransfer_mult(const or_mg_level *c, const or_mg_level *f, const double *x, double *y);
void or_ptransfer_mult_transpose(const or_mg_level *c, const or_mg_level *f, const double *x,
                                 double *y);
/* linalg/solvers.cpp:538-616 (coefficients), 619-656 (Mult) */
void or_chebyshev_coeffs(int order, double lambda, double *c);
void or_chebyshev_mult(const or_mg_level *l, int order, const double *x, double *y);
/* linalg/operator.cpp:886-942 on D^-1 A; start vector: splitmix64(seed) */
double or_power_method(const or_mg_level *l, int steps, double tol, unsigned long long seed);
/* fem/multigrid.cpp:106-239: y = V(1,1)-cycle(x); level 0 solved by CG to
 * coarse_tol (at most coarse_max iterations) */
void or_mg_mult(const or_mg_level *lv, int nl, int order, double coarse_tol, int coarse_max,
                const double *x, double *y);
/* CGSolver::Mult preconditioned by the V-cycle; returns iterations */
int or_mg_pcg(const or_mg_level *lv, int nl, int order, double coarse_tol, int coarse_max,
              const double *b, double *x, double rel_tol, double abs_tol, int max_it,
              double *final_norm, int *converged);

/* DomainLFIntegrator device assembly (fem/integ/lininteg_domain.cpp:22-59,
 * fem/linearform_ext.cpp:20-68): b = R^T (B^T x B^T x B^T)(W f detJ).
 * Q^3 <= 4096. */
void or_domain_lf3d(int ne, int d1d, int q1d, const double *B, const double *W,
                    const double *detJ, const double *f, long c_size, int ndofs,
                    const int *offsets, const int *indices, double *b);

/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int or_num_threads(void);
/* Threads of the following OpenMP regions (timing the CPU baseline at 1 thread). */
void or_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
