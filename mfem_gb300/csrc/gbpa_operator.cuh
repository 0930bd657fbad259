// Operator object shared by the operator and block-solver translation units.
#pragma once
#include "gbpa_dispatch.cuh"
#include "gbpa_tc.cuh"

struct PcgState
{
   double nom, nom0, den, betanom, alpha, beta, r0;
   double rel_tol2, abs_tol2;
   int iter, done, converged, status, final_iter, max_it;
   unsigned int counter_den, counter_beta, counter_init;
   int pad;
};

struct gbpa_operator
{
   // gather map and mask for the element kernels: the pre-masked map when
   // the operator is constrained (no per-gather mask lookup)
   const int *gather() const { return gmap_m ? gmap_m : d.gather_map; }
   const unsigned char *gather_mask() const { return gmap_m ? nullptr : mask; }

   gbpa_ctx *ctx = nullptr;
   gbpa_operator_desc d{};
   unsigned char *mask = nullptr;   // ess mask (ndofs) or null
   unsigned char *emask = nullptr;  // element markers: 1 = the element contributes (null: all do)
   int *gmap_m = nullptr;           // with ess or element markers: gather map with the ess slots and
                                    // every slot of an unmarked element set to GBPA_GATHER_SKIP
   void *yE = nullptr;              // E-vector scratch in the operator's precision
   float2 *qd2 = nullptr;           // GBPA_F64X2: qdata split into (hi, lo) floats
   // tensor-core layout (FP32 diffusion): split Kronecker tables and the
   // per-element output scale; null when the operator was created without it
   gbpa::tc::Tables *tct = nullptr;
   float *tc_qscale = nullptr;
   float *tc_qdata = nullptr;       // qdata in the kernel's tile layout
   // PCG workspace (vectors in the operator's precision)
   void *r = nullptr, *dv = nullptr, *z = nullptr;
   double *partials = nullptr;      // per-block partial sums (PCG_GRID entries x 2)
   PcgState *state = nullptr;
   int64_t ws_n = 0;
   cudaGraphExec_t graph = nullptr;
   const void *graph_x = nullptr, *graph_dinv = nullptr;
   // mixed-precision helpers (FP64 vectors)
   double *r64 = nullptr, *t64 = nullptr;
   // block (multi right-hand side) scratch: E-vector for nrhs interleaved
   void *yEb = nullptr;
   int yEb_nrhs = 0;
   // FP32 block diffusion on the tensor cores, prepared for tcb_nrhs vectors:
   // split Kronecker tables, per-element output scales, qdata in the block
   // kernel's tile layout
   gbpa::tc::Tables *tcb = nullptr;
   float *tcb_qscale = nullptr;
   float *tcb_qdata = nullptr;
   int tcb_nrhs = 0;
   // host-buffer Mult: device staging for pageable x / y (2 L-vectors)
   void *stage = nullptr;
   // gbpa_operator_create_host: the device copies of the descriptor's arrays
   void *owned = nullptr;
};

namespace gbpa
{
// FP32 Jacobi-PCG (CGSolver semantics, zero initial guess) on an FP32 operator.
int pcg_solve_f32(gbpa_operator *A, const float *dinv, const float *b, float *x, double rel_tol,
                  double abs_tol, int max_it, gbpa_solve_info *info);
} // namespace gbpa
