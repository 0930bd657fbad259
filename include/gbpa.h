/* gbpa.h -- GB300-native partial-assembly H1 operator library (C ABI).
 *
 * Drop-in device kernels for MFEM's partial-assembly (PA) H1 path:
 * ElementRestriction gather/scatter, geometric factors, diffusion/mass
 * quadrature-data setup, the sum-factorised 3D diffusion/mass applies and
 * their Jacobi diagonals, and the PCG vector kernels. The reference call site
 * each entry point replaces is cited beside it (paths inside the MFEM tree).
 *
 * Conventions
 *  - Every pointer argument is a DEVICE pointer unless the comment says
 *    "host". Ownership stays with the caller; the library allocates only its
 *    own scratch, which lives in the context.
 *  - Layouts are MFEM's column-major ones:
 *      B, G   (Q, D)                B[q + Q*d];  Bt, Gt (D, Q)
 *      W      (Q, Q, Q)
 *      J      (Q, Q, Q, 3, 3, NE)   J(qx,qy,qz,row,col,e) = d x_row / d xi_col
 *      detJ   (Q^3, NE)
 *      qdata  diffusion (Q, Q, Q, S, NE), S = 6 (symmetric, entries
 *             11,12,13,22,23,33) or 9 (nonsymmetric, row-major 3x3);
 *             mass (Q, Q, Q, NE)
 *      E-vector (D, D, D, NE); L-vector (ndofs) -- vdim = 1 unless stated.
 *  - The return value is GBPA_SUCCESS (0) or a negative GBPA_ERR_* code.
 *    Nothing aborts inside the library; kernels that detect a data error
 *    (non-finite scalar in PCG, zero diagonal) set a sticky flag that
 *    gbpa_get_error_flags() reads and clears.
 *  - Work is enqueued on the context's stream; calls return without waiting
 *    unless they produce a host-visible result (dots, solver statistics).
 */
#ifndef GBPA_H
#define GBPA_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define GBPA_VERSION 10000

enum gbpa_status
{
   GBPA_SUCCESS = 0,
   GBPA_ERR_INVALID_ARGUMENT = -1,
   GBPA_ERR_UNSUPPORTED = -2,  /* (D, Q) outside 1..16, vdim > 3, ... */
   GBPA_ERR_CUDA = -3,         /* a CUDA runtime call failed */
   GBPA_ERR_NOT_FINITE = -4,   /* PCG produced a non-finite scalar */
   GBPA_ERR_ZERO_DIAGONAL = -5,
   GBPA_ERR_NOT_CONVERGED = -6,
   GBPA_ERR_TIMEOUT = -7,
   GBPA_ERR_OUT_OF_MEMORY = -8,
   GBPA_ERR_INDEX = -9         /* an index map entry out of range */
};

/* Sticky device-side error flags (bit mask). */
enum gbpa_error_flag
{
   GBPA_FLAG_NOT_FINITE = 1,
   GBPA_FLAG_ZERO_DIAGONAL = 2,
   GBPA_FLAG_INDEX = 4,
   GBPA_FLAG_INDEFINITE = 8,
   GBPA_FLAG_TIMEOUT = 16      /* a bounded device wait ran out */
};

typedef struct gbpa_ctx *gbpa_ctx_t;

/* ------------------------------------------------------------ context */
/* Replaces Device("cuda") configuration: general/device.cpp:191,443-453. */
int gbpa_version(void);
const char *gbpa_error_string(int status);
int gbpa_create(gbpa_ctx_t *ctx, int device);
int gbpa_destroy(gbpa_ctx_t ctx);
/* Use `stream` (a cudaStream_t) for all later work; NULL restores the
 * context's own non-blocking stream. */
int gbpa_set_stream(gbpa_ctx_t ctx, void *stream);
void *gbpa_get_stream(gbpa_ctx_t ctx);
int gbpa_synchronize(gbpa_ctx_t ctx);
/* host out: flags; clears the device flags. */
int gbpa_get_error_flags(gbpa_ctx_t ctx, int *flags);
/* Number of kernels this context has launched (for launch accounting). */
int64_t gbpa_launch_count(gbpa_ctx_t ctx);

/* -------------------------------------------------- element restriction */
/* ElementRestriction constructor, fem/restriction.cpp:26-114 (host arrays).
 * elem_dofs: element-to-dof table J array (ne x dof, signed, native order);
 * dof_map: lexicographic-to-native map of the element (may be NULL for
 * native ordering). Outputs (host): offsets[ndofs+1], indices[ne*dof],
 * gather_map[ne*dof]. Bit-identical to the reference's maps. */
int gbpa_restriction_build(int ne, int dof, int ndofs, const int *elem_dofs,
                           const int *dof_map, int *offsets, int *indices,
                           int *gather_map);
/* Same construction on the device (all pointers device); gbpa-owned scratch. */
int gbpa_restriction_build_device(gbpa_ctx_t ctx, int ne, int dof, int ndofs,
                                  const int *elem_dofs, const int *dof_map,
                                  int *offsets, int *indices, int *gather_map);
/* ElementRestriction::Mult, fem/restriction.cpp:116-136:
 * y(i%nd, c, i/nd) = +-x(gather_map[i], c). byvdim: L-vector ordering. */
int gbpa_restriction_mult(gbpa_ctx_t ctx, int ne, int nd, int vdim, int byvdim,
                          int ndofs, const int *gather_map, const double *x,
                          double *y);
/* ElementRestriction::AbsMult, fem/restriction.cpp:138-157. */
int gbpa_restriction_abs_mult(gbpa_ctx_t ctx, int ne, int nd, int vdim,
                              int byvdim, int ndofs, const int *gather_map,
                              const double *x, double *y);
/* ElementRestriction::MultTranspose / AddMultTranspose,
 * fem/restriction.cpp:159-201 (add != 0 accumulates into y). Deterministic:
 * each L-dof sums its E-entries in CSR order, as the reference does. */
int gbpa_restriction_mult_transpose(gbpa_ctx_t ctx, int ne, int nd, int vdim,
                                    int byvdim, int ndofs, const int *offsets,
                                    const int *indices, const double *x,
                                    double *y, int add);
/* ElementRestriction::AbsMultTranspose, fem/restriction.cpp:203-228. */
int gbpa_restriction_abs_mult_transpose(gbpa_ctx_t ctx, int ne, int nd,
                                        int vdim, int byvdim, int ndofs,
                                        const int *offsets, const int *indices,
                                        const double *x, double *y);

/* ---------------------------------------------------- geometric factors */
/* GeometricFactors::Compute (JACOBIANS), mesh/mesh.cpp:15445-15500 with
 * QuadratureInterpolator derivatives, fem/qinterp/grad.hpp:233-376:
 * J (Q,Q,Q,3,3,NE) from the lexicographic nodes E-vector X (Dg,Dg,Dg,3,NE)
 * and the nodal basis tables Bg, Gg (Q, Dg). */
int gbpa_geom_jacobians3d(gbpa_ctx_t ctx, int ne, int dg, int q1d,
                          const double *Bg, const double *Gg, const double *X,
                          double *J);
/* DETERMINANTS, fem/qinterp/det.hpp:253-330: detJ (Q^3, NE). */
int gbpa_geom_determinants3d(gbpa_ctx_t ctx, int ne, int dg, int q1d,
                             const double *Bg, const double *Gg,
                             const double *X, double *detJ);
/* COORDINATES, fem/qinterp/eval.hpp: physical coordinates of the quadrature
 * points, layout (Q^3, 3, NE). */
int gbpa_geom_coordinates3d(gbpa_ctx_t ctx, int ne, int dg, int q1d,
                            const double *Bg, const double *X, double *XQ);
/* Coefficient projection at the quadrature points on the device, replacing
 * the host loop of Coefficient::Project(QuadratureFunction&) /
 * CoefficientVector::Project (fem/coefficient.cpp:52-72,2058-2076) for the
 * lognormal field kappa(x) = exp(sum_m amp cos(2 pi k_m . x + phi_m)) that the
 * precision and combined forms use: out (nq, NE) from the physical
 * coordinates XQ (nq, 3, NE) of gbpa_geom_coordinates3d (nq = Q^3).
 * k (host, 3*nmodes integers), phi (host, nmodes), nmodes <= GBPA_MAX_MODES. */
#define GBPA_MAX_MODES 64
int gbpa_coefficient_lognormal3d(gbpa_ctx_t ctx, int ne, int nq, const double *XQ,
                                 int nmodes, const int *k, const double *phi,
                                 double amp, double *out);

/* ------------------------------------------------------------ diffusion */
/* PADiffusionSetup3D, fem/integ/bilininteg_diffusion_kernels.cpp:262-386.
 * coeff_dim: 1 (scalar), 3 (vector/diagonal), 6 (symmetric matrix),
 * 9 (nonsymmetric matrix, transposed as CoefficientVector::ProjectTranspose
 * stores it). c_size == coeff_dim means a constant coefficient, else
 * c_size == coeff_dim*Q^3*NE. Output D has S = (coeff_dim == 9 ? 9 : 6). */
int gbpa_diffusion_setup3d(gbpa_ctx_t ctx, int ne, int q1d, int coeff_dim,
                           const double *W, const double *J, const double *C,
                           int64_t c_size, double *D);
/* Fused geometric factors + setup: J is evaluated from the nodes at each
 * quadrature point and consumed in registers (never stored). */
int gbpa_diffusion_setup3d_nodes(gbpa_ctx_t ctx, int ne, int dg, int q1d,
                                 int coeff_dim, const double *W,
                                 const double *Bg, const double *Gg,
                                 const double *X, const double *C,
                                 int64_t c_size, double *D);
/* DiffusionIntegrator::AddMultPA, fem/integ/bilininteg_diffusion_pa.cpp:41-93
 * (kernels fem/integ/bilininteg_diffusion_kernels.hpp:796-1215):
 * y_E += A_e x_E. Bt/Gt may be NULL (B/G are used transposed). */
int gbpa_diffusion_apply3d(gbpa_ctx_t ctx, int ne, int symm, int d1d, int q1d,
                           const double *B, const double *G, const double *Bt,
                           const double *Gt, const double *D, const double *x,
                           double *y);
int gbpa_diffusion_apply3d_f32(gbpa_ctx_t ctx, int ne, int symm, int d1d,
                               int q1d, const float *B, const float *G,
                               const float *D, const float *x, float *y);
/* DiffusionIntegrator::AssembleDiagonalPA, fem/integ/bilininteg_diffusion_pa.cpp:23-38
 * (kernels fem/integ/bilininteg_diffusion_kernels.hpp:268-485): y_E += diag. */
int gbpa_diffusion_diagonal3d(gbpa_ctx_t ctx, int ne, int symm, int d1d,
                              int q1d, const double *B, const double *G,
                              const double *D, double *y);

/* ----------------------------------------------------------------- mass */
/* MassIntegrator::AssemblePA setup, fem/integ/bilininteg_mass_pa.cpp:73-89:
 * D = W * c * detJ (by_val) or W * c / detJ. c_size 1 = constant. */
int gbpa_mass_setup3d(gbpa_ctx_t ctx, int ne, int nq, const double *W,
                      const double *detJ, const double *C, int64_t c_size,
                      int by_val, double *D);
/* MassIntegrator::AddMultPA, fem/integ/bilininteg_mass_pa.cpp:151-205. */
int gbpa_mass_apply3d(gbpa_ctx_t ctx, int ne, int d1d, int q1d,
                      const double *B, const double *Bt, const double *D,
                      const double *x, double *y);
int gbpa_mass_apply3d_f32(gbpa_ctx_t ctx, int ne, int d1d, int q1d,
                          const float *B, const float *D, const float *x,
                          float *y);
/* MassIntegrator::AssembleDiagonalPA, fem/integ/bilininteg_mass_pa.cpp:138-149. */
int gbpa_mass_diagonal3d(gbpa_ctx_t ctx, int ne, int d1d, int q1d,
                         const double *B, const double *D, double *y);

/* ------------------------------------------- L-vector PA operator (fused) */
/* PABilinearFormExtension::Mult for one domain integrator,
 * fem/bilinearform_ext.cpp:487-564 (restriction -> AddMultPA -> transpose),
 * optionally wrapped in ConstrainedOperator (linalg/operator.cpp:526-661,
 * DIAG_ONE). The gather of x is fused into the apply kernel; the scatter is
 * the deterministic CSR sum (or atomic adds, see GBPA_SCATTER_ATOMIC). */
enum gbpa_kind { GBPA_DIFFUSION = 0, GBPA_MASS = 1 };
/* GBPA_F64X2: FP64 data (qdata, B, G, x, y all FP64) applied with
 * double-float arithmetic on the FP32 pipes -- each value is an unevaluated
 * sum of two floats with exact product/sum error terms (~2^-44 relative per
 * operation) -- because GB300's FP32 rate is ~58x its FP64 rate. The operator
 * keeps an internal (hi, lo) float copy of qdata (same bytes as FP64). */
enum gbpa_precision { GBPA_F64 = 0, GBPA_F32 = 1, GBPA_F64X2 = 2 };
/* GBPA_SCATTER_CSR: deterministic row sums in the reference's order (default).
 * GBPA_SCATTER_ATOMIC: the element kernel adds its results into y through the
 * gather map (no E-vector); reproducible to rounding only; y must not alias x.
 * The block and batched solvers always use the CSR scatter. */
enum gbpa_scatter { GBPA_SCATTER_CSR = 0, GBPA_SCATTER_ATOMIC = 1 };

typedef struct gbpa_operator_desc
{
   int kind;            /* gbpa_kind */
   int precision;       /* gbpa_precision of qdata/B/G and of x, y in mult */
   int ne, ndofs, d1d, q1d;
   int symm;            /* diffusion: 1 if S = 6 */
   const void *B, *G;   /* (Q, D) in `precision` */
   const void *qdata;   /* in `precision` */
   const int *gather_map, *offsets, *indices;
   const int *ess;      /* essential (constrained) dofs, may be NULL */
   int n_ess;
   int scatter;         /* gbpa_scatter */
} gbpa_operator_desc;

typedef struct gbpa_operator *gbpa_operator_t;

int gbpa_operator_create(gbpa_ctx_t ctx, const gbpa_operator_desc *desc,
                         gbpa_operator_t *op);
/* gbpa_operator_create with every array of the descriptor (B, G, qdata,
 * gather_map, offsets, indices, ess) in HOST memory: the library keeps
 * device copies, freed by gbpa_operator_destroy. For hosts whose arrays
 * live in host memory -- an MFEM built without CUDA, whose
 * PABilinearFormExtension then forwards Mult to gbpa_operator_mult_host
 * (integration/gbpa_shim.cpp). */
int gbpa_operator_create_host(gbpa_ctx_t ctx, const gbpa_operator_desc *desc,
                              gbpa_operator_t *op);
int gbpa_operator_destroy(gbpa_operator_t op);
/* y = A x (L-vectors, the descriptor's precision). With ess dofs:
 * y = A (x with ess zeroed), then y[ess] = x[ess]. */
int gbpa_operator_mult(gbpa_operator_t op, const void *x, void *y);
/* gbpa_operator_mult with x and y in HOST memory; returns when y holds the
 * result. Replaces the host<->device transfers MFEM's memory manager makes
 * around a device Mult of host-valid Vectors (Vector::Read ->
 * MemoryManager::Read_, general/mem_manager.cpp:1109-1131, copies x to the
 * device; Vector::HostRead of y copies it back). Pinned buffers (cudaHostAlloc,
 * cudaHostRegister) are device-mapped: the element kernel gathers x and the
 * scatter writes y through them directly over the host-device link (NVLink-C2C
 * on Grace-Blackwell), so the transfers run inside the apply instead of
 * before and after it. Pageable buffers are staged through device scratch
 * with cudaMemcpyAsync. */
int gbpa_operator_mult_host(gbpa_operator_t op, const void *x, void *y);
/* Element part of the operator alone: yE = A_e (R x) with the gather of x
 * fused into the sum-factorised apply (ElementRestriction::Mult followed by
 * AddMultPA on a zeroed E-vector, fem/bilinearform_ext.cpp:530-546). yE is
 * an E-vector (D, D, D, NE) in the descriptor's precision. */
int gbpa_operator_apply_element(gbpa_operator_t op, const void *x, void *yE);
/* Domain-integrator element markers: PABilinearFormExtension::
 * AddMultWithMarkers with AddWithMarkers_ (fem/bilinearform_ext.cpp:530-550,
 * 753-774, 807-847) and the marked diagonal (:405-440). Element e contributes
 * to Mult, the PCG solves and AssembleDiagonal iff attributes[e] > 0 and
 * markers[attributes[e] - 1] != 0 (BilinearForm::AddDomainIntegrator(integ,
 * elem_marker) with the mesh's element attributes). attributes: device
 * int[ne]; markers: device int[n_markers], one per attribute. An attribute
 * above n_markers returns GBPA_ERR_INDEX and leaves every element active.
 * attributes == NULL removes the markers (every element contributes). The
 * arrays are read during the call only. */
int gbpa_operator_set_element_markers(gbpa_operator_t op, const int *attributes,
                                      const int *markers, int n_markers);
/* BilinearForm::AssembleDiagonal (PA), fem/bilinearform_ext.cpp:370-454,
 * with ConstrainedOperator::AssembleDiagonal DIAG_ONE when ess is set.
 * diag is always FP64. */
int gbpa_operator_assemble_diagonal(gbpa_operator_t op, double *diag);

/* ------------------------------------------------- allocation-free apply */
/* No counterpart in the reference. Computes y = R^T A_e R x for FP64
 * diffusion -- what gbpa_operator_mult computes for an unconstrained FP64
 * diffusion operator -- for callers that cannot allocate device memory: an
 * application whose device memory is owned by its own pool allocator, or a
 * path that must not trigger the device synchronisation cudaMalloc/cudaFree
 * can cause. The E-vector scratch is a fixed static device array of
 * GBPA_NOALLOC_MAX_EVEC doubles (16 MiB, held by every GPU that loads the
 * library until the process exits); ne*d1d^3 beyond it returns
 * GBPA_ERR_UNSUPPORTED. Work goes on `stream` (NULL: the legacy default
 * stream). All calls share the scratch, so calls that overlap on the GPU race:
 * serialise them. The first call on each device looks up the scratch's device
 * address and keeps it; make it before any stream capture, and do not use this
 * entry point after a cudaDeviceReset of that device (the kept address belonged
 * to the old context). (D, Q) beyond 16 returns GBPA_ERR_UNSUPPORTED. */
#define GBPA_NOALLOC_MAX_EVEC (1 << 21)
int gbpa_diffusion_mult_noalloc(void *stream, int ne, int ndofs, int d1d, int q1d,
                                int symm, const double *B, const double *G,
                                const double *qdata, const int *gather_map,
                                const int *offsets, const int *indices,
                                const double *x, double *y);

/* -------------------------------------------------------- vector kernels */
/* Vector::operator* (linalg/vector.cpp:1079-1106) with reduce()
 * (general/reducers.hpp:531-594): host out *result. Warp-shuffle tree,
 * fixed order (deterministic for a given n). */
int gbpa_vec_dot(gbpa_ctx_t ctx, int64_t n, const double *x, const double *y,
                 double *result);
/* add(x, a, y, z): z = x + a*y (linalg/vector.cpp:414-600). */
int gbpa_vec_add(gbpa_ctx_t ctx, int64_t n, const double *x, double a,
                 const double *y, double *z);
/* OperatorJacobiSmoother::Setup, linalg/solvers.cpp:401-425:
 * dinv = damping/diag, dinv[ess] = damping. Zero diagonal -> error status. */
int gbpa_jacobi_setup(gbpa_ctx_t ctx, int64_t n, const double *diag,
                      const int *ess, int n_ess, double damping, double *dinv);

/* ------------------------------------------------------------------ PCG */
typedef struct gbpa_solve_info
{
   int iterations;       /* CGSolver::GetNumIterations */
   int converged;        /* CGSolver::GetConverged */
   double initial_norm;  /* sqrt((B r0, r0)) */
   double final_norm;    /* sqrt((B r, r)) at exit, CGSolver::GetFinalNorm */
   double true_rel_residual; /* ||b - A x|| / ||b|| evaluated in FP64 */
   int outer_iterations; /* mixed-precision form: defect-correction steps */
   int inner_iterations; /* mixed-precision form: total FP32 PCG iterations */
   double seconds;       /* device time of the solve */
} gbpa_solve_info;

/* CGSolver::Mult, linalg/solvers.cpp:869-1050, preconditioned by
 * OperatorJacobiSmoother::Mult (linalg/solvers.cpp:427-452, non-iterative):
 * the whole iteration runs on the device (no host round trip per dot); the
 * host polls the convergence flag every `check_every` iterations from a
 * captured CUDA graph. iterative_mode != 0 starts from x. Same stopping
 * rule as the reference: (B r, r) <= max(rel_tol^2 (B r0, r0), abs_tol^2). */
int gbpa_pcg_solve(gbpa_operator_t A, const double *dinv, const double *b,
                   double *x, double rel_tol, double abs_tol, int max_it,
                   int iterative_mode, gbpa_solve_info *info);

/* Mixed-precision form: FP64 defect correction around FP32 Jacobi-PCG inner
 * solves. A64 is the FP64 operator (true residual r = b - A x in FP64), A32
 * its FP32 twin (same maps, FP32 qdata/B/G). Outer loop stops when
 * ||b - A64 x|| <= outer_rel_tol ||b||; each inner solve stops at relative
 * preconditioned residual inner_rel_tol. dinv32 is FP32. */
int gbpa_pcg_solve_mixed(gbpa_operator_t A64, gbpa_operator_t A32,
                         const float *dinv32, const double *b, double *x,
                         double outer_rel_tol, double inner_rel_tol,
                         int max_outer, int max_inner, gbpa_solve_info *info);
/* Mixed precision with reliable updates (no counterpart in the reference; it
 * replaces the same CGSolver::Mult call as gbpa_pcg_solve): ONE FP32
 * Jacobi-PCG on A32 whose iterated residual is replaced by the true FP64
 * residual b - A64 x whenever its preconditioned norm has dropped by `delta`
 * (0 < delta < 1, e.g. 0.1) since the last replacement; the search direction
 * keeps its history, so no Krylov space is discarded. Stops when
 * ||b - A64 x|| <= rel_tol ||b|| (FP64, 2-norm) or after max_it FP32
 * iterations. info: iterations = FP32 iterations, outer_iterations =
 * residual replacements. x starts from zero. */
int gbpa_pcg_solve_mixed_reliable(gbpa_operator_t A64, gbpa_operator_t A32,
                                  const float *dinv32, const double *b, double *x,
                                  double rel_tol, double delta, int max_it,
                                  gbpa_solve_info *info);

/* ------------------------------------------- several right-hand sides */
/* R = nrhs right-hand sides stored interleaved (v[i*R + r]), R in {1, 2, 4,
 * 8}; diffusion operators only. The block apply reads each element's qdata
 * once for all R vectors (BilinearForm::Mult applied to R vectors,
 * fem/bilinearform_ext.cpp:487-564). */
int gbpa_operator_mult_block(gbpa_operator_t op, int nrhs, const void *x, void *y);
/* R independent CGSolver::Mult recurrences (linalg/solvers.cpp:869-1050),
 * one set of scalars and one stopping test per right-hand side, sharing the
 * block apply. FP64 (or F64X2) operator; info has nrhs entries. */
int gbpa_pcg_solve_block(gbpa_operator_t A, int nrhs, const double *dinv,
                         const double *b, double *x, double rel_tol,
                         double abs_tol, int max_it, gbpa_solve_info *info);
/* Mixed precision per right-hand side: FP32 block PCG inner solves inside
 * FP64 defect correction with FP64 true residuals (b - A64 x), until every
 * right-hand side reaches outer_rel_tol. */
int gbpa_pcg_solve_block_mixed(gbpa_operator_t A64, gbpa_operator_t A32,
                               int nrhs, const float *dinv32, const double *b,
                               double *x, double outer_rel_tol,
                               double inner_rel_tol, int max_outer,
                               int max_inner, gbpa_solve_info *info);
/* Block form of gbpa_pcg_solve_mixed_reliable: one FP32 block PCG whose
 * residuals are replaced by the true FP64 block residual once every
 * right-hand side still running has dropped by `delta` since its last
 * replacement. info[r]: iterations = FP32 iterations, outer_iterations =
 * replacements; each right-hand side stops on its own true FP64 residual. */
int gbpa_pcg_solve_block_mixed_reliable(gbpa_operator_t A64, gbpa_operator_t A32,
                                        int nrhs, const float *dinv32,
                                        const double *b, double *x, double rel_tol,
                                        double delta, int max_it,
                                        gbpa_solve_info *info);

/* ---------------------------------------------------------- batched PCG */
/* Batching form: many independent Dirichlet problems of uneven size and
 * order, solved together. Each problem owns its maps, qdata and vectors
 * (device pointers inside the descriptor array, which is itself host
 * memory). All problems advance in lockstep; a per-problem converged mask
 * stops finished problems. Each problem follows CGSolver::Mult with
 * OperatorJacobiSmoother (linalg/solvers.cpp:869-1050) on its
 * ConstrainedOperator-wrapped PA diffusion operator; no single reference
 * entry point solves several problems at once. FP64. */
typedef struct gbpa_problem_desc
{
   int ne, ndofs, d1d, q1d;
   const double *B, *G, *qdata;          /* symmetric diffusion qdata */
   const int *gather_map, *offsets, *indices;
   const int *ess; int n_ess;
   const double *dinv;                   /* Jacobi inverse diagonal */
   const double *b;
   double *x;
} gbpa_problem_desc;

int gbpa_batched_pcg_solve(gbpa_ctx_t ctx, int nprob,
                           const gbpa_problem_desc *probs, double rel_tol,
                           double abs_tol, int max_it, int *iterations,
                           int *converged, double *final_norms,
                           double *seconds);
/* Same, with the element arithmetic chosen: GBPA_F64 (as above) or
 * GBPA_F64X2 (FP64 data, double-float arithmetic on the FP32 pipes; the
 * library splits each problem's qdata into its workspace). */
int gbpa_batched_pcg_solve_precision(gbpa_ctx_t ctx, int nprob,
                                     const gbpa_problem_desc *probs,
                                     int precision, double rel_tol,
                                     double abs_tol, int max_it,
                                     int *iterations, int *converged,
                                     double *final_norms, double *seconds);

/* How the batched iterations are scheduled on the GPU.
 *  GBPA_BATCH_GRAPH       each PCG iteration is a few launches that cover
 *                         all active problems (one grouped element-apply
 *                         launch per order, with that order's compile-time
 *                         kernel, then the vector phases), K iterations
 *                         captured in a CUDA graph; the work tables are
 *                         compacted as problems converge. Orders up to
 *                         d1d, q1d <= 10. The default.
 *  GBPA_BATCH_PERSISTENT  one cooperative persistent launch for the whole
 *                         solve, grid-wide barriers between the phases and
 *                         one runtime-size element kernel (p <= 6). */
enum gbpa_batch_schedule { GBPA_BATCH_GRAPH = 0, GBPA_BATCH_PERSISTENT = 1 };
int gbpa_batched_pcg_solve_ex(gbpa_ctx_t ctx, int nprob,
                              const gbpa_problem_desc *probs, int precision,
                              int schedule, double rel_tol, double abs_tol,
                              int max_it, int *iterations, int *converged,
                              double *final_norms, double *seconds);

/* ------------------------------------------------------ vector diffusion */
/* VectorDiffusionIntegrator::AssemblePA, 3D, scalar or vector coefficient
 * (fem/integ/bilininteg_vecdiffusion_pa.cpp:68-276): for each component c of
 * a vdim-component H1 space, the symmetric diffusion qdata scaled by the
 * coefficient component (coeff_vdim 1: the same scalar for every
 * component; coeff_vdim = vdim: C_c). C laid out (coeff_vdim, Q^3, NE),
 * c_size coeff_vdim (constant) or coeff_vdim Q^3 NE. D: (Q^3, 6, vdim, NE),
 * which fits in the reference's pa_data (Q^3 9 vdim NE). coeff_vdim 9 (vdim
 * 3) is a matrix coefficient, C (9, Q^3, NE) as CoefficientVector::
 * ProjectTranspose stores it: block b of D (layout (Q^3, 6, NE, 9)) is the
 * geometric factor times C(map[b]), map = {0,3,6,1,4,7,2,5,8} (:119-130,
 * 213-272); apply it with gbpa_vector_diffusion_apply3d_coeff. */
int gbpa_vector_diffusion_setup3d(gbpa_ctx_t ctx, int ne, int q1d, int vdim,
                                  int coeff_vdim, const double *W,
                                  const double *J, const double *C,
                                  int64_t c_size, double *D);
/* VectorDiffusionIntegrator::AddMultPA, 3D (kernel
 * fem/integ/bilininteg_vecdiffusion_pa.hpp:96-163): y_E += A_e x_E on the
 * (D^3, vdim, NE) E-vectors of the vector space's element restriction. */
int gbpa_vector_diffusion_apply3d(gbpa_ctx_t ctx, int ne, int vdim, int d1d,
                                  int q1d, const double *B, const double *G,
                                  const double *D, const double *x, double *y);
/* The same with the coefficient's vdim, as ApplyPAKernels::Run receives it
 * (fem/integ/bilininteg_vecdiffusion_pa.cpp:276-330): coeff_vdim 1 or vdim as
 * above; coeff_vdim 9 with vdim 3 is the matrix coefficient
 * (VectorDiffusionIntegrator(MatrixCoefficient&), :64-68,119-130), whose
 * components couple: y_j += G^T D_(j+3i) G x_i, with D written by
 * gbpa_vector_diffusion_setup3d(coeff_vdim 9) in the block-major layout
 * (Q^3, 6, NE, 9) (it fits the reference's pa_data, Q^3 * 9 * 9 * NE). */
int gbpa_vector_diffusion_apply3d_coeff(gbpa_ctx_t ctx, int ne, int vdim, int coeff_vdim,
                                        int d1d, int q1d, const double *B,
                                        const double *G, const double *D,
                                        const double *x, double *y);

/* VectorMassIntegrator::AssemblePA / AddMultPA, 3D, scalar or vector
 * coefficient (fem/integ/bilininteg_vecmass_pa.cpp:21-210): D (Q^3,
 * coeff_vdim, NE) = C_k W detJ, the reference's own layout; the apply runs
 * the scalar mass operator per component on the (D^3, vdim, NE) E-vectors.
 * A matrix coefficient (vdim 3, coeff_vdim 9, C (9, Q^3, NE) as
 * CoefficientVector::ProjectTranspose stores it) couples the components:
 * D is then block-major (Q^3, NE, 9), block 3c+d = C(3c+d) W detJ, and the
 * apply adds y_c += B^T D_(3c+d) B x_d (fem/integ/bilininteg_vecmass_pa.hpp:
 * 157-170). */
int gbpa_vector_mass_setup3d(gbpa_ctx_t ctx, int ne, int q1d, int vdim,
                             int coeff_vdim, const double *W, const double *J,
                             const double *C, int64_t c_size, double *D);
int gbpa_vector_mass_apply3d(gbpa_ctx_t ctx, int ne, int vdim, int coeff_vdim,
                             int d1d, int q1d, const double *B,
                             const double *D, const double *x, double *y);

/* ---------------------------------------------------------- linear form */
/* DomainLFIntegrator::AssembleDevice + LinearFormExtension::Assemble
 * (fem/integ/lininteg_domain.cpp:22-59, DLFEvalAssemble3D in
 * fem/integ/lininteg_domain_kernels.hpp:164-..., fem/linearform_ext.cpp:
 * 20-68): b = R^T (B^T x B^T x B^T)(W f detJ) for one DomainLFIntegrator
 * over all elements, b overwritten. B (Q, D) and W (Q^3) at the linear
 * form's rule (the reference's default: order 2p, Q = p + 1), detJ (Q^3,
 * NE) at that rule, f: coeff_size 1 (constant) or Q^3 NE values (the
 * CoefficientVector at the rule's physical points). offsets/indices: the
 * lexicographic restriction's CSR maps. */
int gbpa_domain_lf3d(gbpa_ctx_t ctx, int ne, int d1d, int q1d,
                     const double *B, const double *W, const double *detJ,
                     const double *coeff, int64_t coeff_size, int ndofs,
                     const int *offsets, const int *indices, double *b);

/* ---------------------------------------------------------- p-multigrid */
/* p-multigrid preconditioning around the PA diffusion operator, the
 * structure of the reference's examples/ex26.cpp. Levels are operators
 * (gbpa_operator_create), borrowed, never freed by these objects: all with
 * FP64 vectors (precision GBPA_F64 or GBPA_F64X2) or all GBPA_F32 (float
 * vectors; the V-cycle then runs in FP32 as a preconditioner of the FP64
 * CG). Vector arguments are in the levels' type. */

/* p-refinement transfer between two H1 spaces on the same mesh
 * (TensorProductPRefinementTransferOperator, fem/transfer.cpp:2620-2990;
 * FiniteElementSpace::GetTransferOperator picks it for tensor H1 spaces of
 * different orders, fem/transfer.cpp:2195-2216). The maps are the two
 * spaces' lexicographic ElementRestriction maps (device memory, borrowed);
 * Bi (d1d_f, d1d_c), host memory, column-major: the coarse Lagrange basis
 * at the fine element's lexicographic nodes. d1d <= 10. precision:
 * GBPA_F64 (double vectors) or GBPA_F32 (float vectors). */
typedef struct gbpa_ptransfer *gbpa_ptransfer_t;
int gbpa_ptransfer_create(gbpa_ctx_t ctx, int ne, int d1d_c, int ndofs_c,
                          const int *gather_map_c, const int *offsets_c,
                          const int *indices_c, int d1d_f, int ndofs_f,
                          const int *gather_map_f, const int *offsets_f,
                          const int *indices_f, const double *Bi,
                          int precision, gbpa_ptransfer_t *out);
int gbpa_ptransfer_destroy(gbpa_ptransfer_t T);
/* TransferOperator::Mult: y_f = P x_c (prolongation) */
int gbpa_ptransfer_mult(gbpa_ptransfer_t T, const void *xc, void *yf);
/* TransferOperator::MultTranspose: y_c = P^T x_f */
int gbpa_ptransfer_mult_transpose(gbpa_ptransfer_t T, const void *xf,
                                  void *yc);

/* OperatorChebyshevSmoother (linalg/solvers.cpp:455-660) for the
 * constrained operator A with its unconstrained diagonal `diag` (device).
 * max_eig > 0: the given estimate of the largest eigenvalue of D^-1 A
 * (the constructor at solvers.cpp:455-469); max_eig <= 0: estimated by
 * PowerMethod::EstimateLargestEigenvalue (linalg/operator.cpp:886-942) with
 * power_iterations steps and tolerance power_tol (the reference's defaults:
 * 10, 1e-8) from a splitmix64 start vector of `seed` (the reference draws
 * it with the C library's rand()). order 1..8. */
typedef struct gbpa_chebyshev *gbpa_chebyshev_t;
int gbpa_chebyshev_create(gbpa_operator_t A, const double *diag, int order,
                          double max_eig, int power_iterations,
                          double power_tol, unsigned long long seed,
                          gbpa_chebyshev_t *out);
int gbpa_chebyshev_destroy(gbpa_chebyshev_t S);
int gbpa_chebyshev_get_max_eig(gbpa_chebyshev_t S, double *max_eig);
int gbpa_chebyshev_mult(gbpa_chebyshev_t S, const void *x, void *y);

/* Multigrid (fem/multigrid.cpp:106-239): V-cycle with one pre- and one
 * post-smoothing step; level 0 (coarsest) solved by CGSolver to
 * coarse_rel_tol in at most coarse_max_it iterations, without a
 * preconditioner (coarse_jacobi = 0: examples/ex26.cpp, 1e-2 and 200) or
 * with the Jacobi smoother of the coarse operator (coarse_jacobi = 1; its
 * diagonal coarse_diag, FP64 device memory, or NULL to assemble it from
 * the coarse operator, which needs FP64 data). ops[0..nlevels),
 * smoothers[1..nlevels) (smoothers[0] unused), prolongations[l] from level
 * l to l+1. */
typedef struct gbpa_multigrid *gbpa_multigrid_t;
int gbpa_multigrid_create(gbpa_ctx_t ctx, int nlevels,
                          const gbpa_operator_t *ops,
                          const gbpa_chebyshev_t *smoothers,
                          const gbpa_ptransfer_t *prolongations,
                          double coarse_rel_tol, int coarse_max_it,
                          int coarse_jacobi, const double *coarse_diag,
                          gbpa_multigrid_t *out);
int gbpa_multigrid_destroy(gbpa_multigrid_t M);
/* MultigridBase::Mult: y = one V-cycle applied to x (zero initial guess) */
int gbpa_multigrid_mult(gbpa_multigrid_t M, const void *x, void *y);
/* CGSolver::Mult (linalg/solvers.cpp:869-1050) on A (FP64 vectors, the
 * finest level's size) preconditioned by M, zero initial guess; with FP32
 * levels the residual is narrowed into the cycle and the correction widened
 * back. info->iterations: outer CG
 * iterations; info->inner_iterations: coarse-level CG iterations summed
 * over all cycles; true_rel_residual is not computed (-1). */
int gbpa_pcg_solve_mg(gbpa_operator_t A, gbpa_multigrid_t M, const double *b,
                      double *x, double rel_tol, double abs_tol, int max_it,
                      gbpa_solve_info *info);

/* --------------------------------------------------------------- tuning */
/* Elements per thread block used by the apply kernels for (kind, precision,
 * d1d, q1d); 0 = library default. The autotuner (python side) sweeps this. */
int gbpa_set_elements_per_block(int kind, int precision, int d1d, int q1d,
                                int nbz);
int gbpa_get_elements_per_block(int kind, int precision, int d1d, int q1d);
/* Thread layout of the gather-fused diffusion or mass apply (the operator
 * path) for (kind, precision, d1d, q1d): GBPA_LAYOUT_SLAB2D (default; block (Q, Q, nbz), one
 * thread per (qx, qy) column, z in registers) or GBPA_LAYOUT_3D (block
 * (Q, Q, Q*nbz), one thread per quadrature point, every contraction through
 * shared memory; compile-time kernels for the (D, Q) pairs the 2D slab
 * specialises, others stay 2D; nbz * q1d <= 64 and nbz * q1d^3 <= 1024), or
 * GBPA_LAYOUT_TC (FP32 diffusion operators only, (d1d, q1d) in (3,4), (4,5),
 * (5,6); nbz ignored): the element contraction as two dense GEMMs per tile of
 * 128 elements on the tcgen05 tensor cores (fp16 hi/lo operand limbs, FP32
 * accumulation). An operator picks up the tensor-core layout when it is
 * selected at operator creation. The autotuner chooses per order. get
 * returns the layout and its nbz. */
enum gbpa_layout { GBPA_LAYOUT_SLAB2D = 0, GBPA_LAYOUT_3D = 1, GBPA_LAYOUT_TC = 2 };
int gbpa_set_apply_layout(int kind, int precision, int d1d, int q1d, int layout,
                          int nbz);
int gbpa_get_apply_layout(int kind, int precision, int d1d, int q1d, int *nbz);
/* The element kernel of the FP32 block diffusion apply
 * (gbpa_operator_mult_block and the block solvers) for (d1d, q1d, nrhs):
 * GBPA_LAYOUT_TC, the tensor-core block kernel (a tile of 128 / nrhs elements
 * times nrhs vectors; the default where one exists: (5,6) and (6,7) with
 * nrhs 8), or GBPA_LAYOUT_SLAB2D, the CUDA-core block kernel. TC where no
 * kernel exists returns GBPA_ERR_UNSUPPORTED. An operator prepares the
 * tensor-core data (tables, scales, re-laid qdata: about the size of its
 * qdata) at its first block apply or block solve with the layout selected. */
int gbpa_set_block_apply_layout(int d1d, int q1d, int nrhs, int layout);
int gbpa_get_block_apply_layout(int d1d, int q1d, int nrhs);

/* ------------------------------------------------ failure-detection test */
/* No counterpart in the reference. Makes one of the library's bounded device
 * waits run out on purpose -- the arrival it waits for never comes -- and
 * reports what the wait reported: which = 0, the persistent batched kernel's
 * grid barrier with one block never arriving (limit: spins); which = 1, the
 * TMA staging mbarrier wait with no copy issued (limit: polls). Returns
 * GBPA_ERR_TIMEOUT when the wait gave up as designed; the kernel has returned
 * and the context stays usable. limit <= 2^26. */
int gbpa_selftest_bounded_wait(gbpa_ctx_t ctx, int which, long long limit);

#ifdef __cplusplus
}
#endif
#endif /* GBPA_H */
