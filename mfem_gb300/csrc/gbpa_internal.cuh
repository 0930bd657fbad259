// Internal declarations shared by the gbpa CUDA translation units.
#pragma once
#include "../../include/gbpa.h"
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <vector>

#define GBPA_MAX_1D 16       // largest D1D / Q1D handled (the generic kernels)
// Gather-map entry that reads as zero: a constrained operator's pre-masked
// copy of the map marks its essential dofs' slots with it, so the gather
// needs no separate mask lookup. Never a valid signed index (-1 - j with
// j <= INT_MAX - 1, since ndofs is an int).
#define GBPA_GATHER_SKIP (-2147483647 - 1)

struct gbpa_ctx
{
   int device = 0;
   int num_sms = 0;
   cudaStream_t own_stream = nullptr;
   cudaStream_t stream = nullptr;
   cudaStream_t capture_stream = nullptr; // private stream for CUDA-graph capture
                                          // (the legacy default stream cannot be captured)
   int *d_flags = nullptr;           // sticky device error flags
   double *h_pinned = nullptr;       // small pinned host staging area (64 doubles)
   double *d_scalars = nullptr;      // small device scalar area (64 doubles)
   unsigned int *d_counter = nullptr;// last-block-done counter for reductions
   double *d_partials = nullptr;     // per-block partial sums (4096 doubles)
   int64_t launches = 0;
   // growable scratch slots (device memory owned by the context)
   struct Slot { void *ptr = nullptr; size_t bytes = 0; };
   std::vector<Slot> slots;
};

namespace gbpa
{
enum ScratchSlot
{
   SLOT_EVEC_A = 0, SLOT_EVEC_B, SLOT_RESTRICT, SLOT_PCG, SLOT_PCG32,
   SLOT_BATCH, SLOT_TMP, SLOT_COUNT
};

void *scratch(gbpa_ctx *ctx, int slot, size_t bytes);   // nullptr on OOM
int check_cuda(cudaError_t e, const char *what);
inline int last_launch(gbpa_ctx *ctx, const char *what)
{
   ctx->launches++;
   return check_cuda(cudaGetLastError(), what);
}
inline unsigned grid_for(int64_t n, int block, int max_blocks = 1 << 20)
{
   int64_t g = (n + block - 1) / block;
   if (g < 1) { g = 1; }
   if (g > max_blocks) { g = max_blocks; }
   return (unsigned)g;
}

// Device time of a stretch of work on a stream: started at construction,
// read by stop(); the events are released on every return path.
struct StreamTimer
{
   cudaEvent_t e0 = nullptr, e1 = nullptr;
   explicit StreamTimer(cudaStream_t s)
   {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, s);
   }
   // milliseconds since construction (waits for the stream's work so far)
   float stop(cudaStream_t s)
   {
      cudaEventRecord(e1, s);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) == cudaSuccess) { cudaEventElapsedTime(&ms, e0, e1); }
      return ms;
   }
   ~StreamTimer()
   {
      if (e0) { cudaEventDestroy(e0); }
      if (e1) { cudaEventDestroy(e1); }
   }
   StreamTimer(const StreamTimer &) = delete;
   StreamTimer &operator=(const StreamTimer &) = delete;
};

// ---------------------------------------------------------------- kernels
// E-vector apply kernels (2D-slab: one thread per (qx,qy) column, z in
// registers, nbz elements per block). gather_map != nullptr: x is an
// L-vector gathered (with sign) through the map; ess_mask zeroes
// constrained dofs on the fly. accumulate (the output mode): 0 y = result,
// 1 y += result (E-vector y), GBPA_OUT_ATOMIC: each E-slot's result is added
// atomically into the L-vector y at the dof the gather map gives it (the
// scatter fused into the apply; y must be zeroed first, constrained slots add
// nothing).
constexpr int GBPA_OUT_ATOMIC = 2;
template <typename T>
int launch_diffusion_apply(gbpa_ctx *ctx, int ne, int symm, int D, int Q,
                           const T *B, const T *G, const T *qd, const T *x,
                           const int *gather_map, const unsigned char *ess_mask,
                           T *y, int accumulate, const int *skip = nullptr);
template <typename T>
int launch_mass_apply(gbpa_ctx *ctx, int ne, int D, int Q, const T *B,
                      const T *qd, const T *x, const int *gather_map,
                      const unsigned char *ess_mask, T *y, int accumulate,
                      const int *skip = nullptr);
template <>
int launch_diffusion_apply<double>(gbpa_ctx *, int, int, int, int, const double *, const double *,
                                   const double *, const double *, const int *,
                                   const unsigned char *, double *, int, const int *);
template <>
int launch_diffusion_apply<float>(gbpa_ctx *, int, int, int, int, const float *, const float *,
                                  const float *, const float *, const int *,
                                  const unsigned char *, float *, int, const int *);
template <>
int launch_mass_apply<double>(gbpa_ctx *, int, int, int, const double *, const double *,
                              const double *, const int *, const unsigned char *, double *, int,
                              const int *);
template <>
int launch_mass_apply<float>(gbpa_ctx *, int, int, int, const float *, const float *,
                             const float *, const int *, const unsigned char *, float *, int,
                             const int *);
// FP64-accurate double-float arithmetic on the FP32 pipes (qdata split into
// float2 (hi, lo) by launch_split_x2).
int launch_diffusion_apply_x2(gbpa_ctx *ctx, int ne, int symm, int D, int Q, const double *B,
                              const double *G, const float2 *qd, const double *x,
                              const int *gather_map, const unsigned char *ess_mask, double *y,
                              int accumulate, const int *skip = nullptr);
int launch_mass_apply_x2(gbpa_ctx *ctx, int ne, int D, int Q, const double *B, const float2 *qd,
                         const double *x, const int *gather_map, const unsigned char *ess_mask,
                         double *y, int accumulate, const int *skip = nullptr);
int launch_split_x2(gbpa_ctx *ctx, int64_t n, const double *a, float2 *b);
// Gather-fused diffusion apply in the 3D thread layout (one translation unit
// per arithmetic); GBPA_ERR_UNSUPPORTED when (D, Q) has no 3D kernel.
int launch_diffusion_3d_f64(gbpa_ctx *ctx, int ne, int symm, int D, int Q, const double *B,
                            const double *G, const double *qd, const double *x, const int *gather_map,
                            const unsigned char *ess_mask, double *y, int mode, const int *skip, int nbz);
int launch_diffusion_3d_f32(gbpa_ctx *ctx, int ne, int symm, int D, int Q, const float *B,
                            const float *G, const float *qd, const float *x, const int *gather_map,
                            const unsigned char *ess_mask, float *y, int mode, const int *skip, int nbz);
int launch_diffusion_3d_x2(gbpa_ctx *ctx, int ne, int symm, int D, int Q, const double *B,
                           const double *G, const float2 *qd, const double *x, const int *gather_map,
                           const unsigned char *ess_mask, double *y, int mode, const int *skip, int nbz);
// The same for the mass apply.
int launch_mass_3d_f64(gbpa_ctx *ctx, int ne, int D, int Q, const double *B, const double *qd, const double *x,
                       const int *gather_map, const unsigned char *ess_mask, double *y, int mode,
                       const int *skip, int nbz);
int launch_mass_3d_f32(gbpa_ctx *ctx, int ne, int D, int Q, const float *B, const float *qd, const float *x,
                       const int *gather_map, const unsigned char *ess_mask, float *y, int mode,
                       const int *skip, int nbz);
int launch_mass_3d_x2(gbpa_ctx *ctx, int ne, int D, int Q, const double *B, const float2 *qd, const double *x,
                      const int *gather_map, const unsigned char *ess_mask, double *y, int mode,
                      const int *skip, int nbz);
// FP64 E-vector mass apply (y += A_e x) where element e reads the qdata of
// element e / qdiv.
int launch_mass_apply_qdiv(gbpa_ctx *ctx, int ne, int D, int Q, const double *B, const double *qd,
                           const double *x, double *y, int qdiv);
int launch_diffusion_diagonal(gbpa_ctx *ctx, int ne, int symm, int D, int Q,
                              const double *B, const double *G,
                              const double *qd, double *y);
int launch_mass_diagonal(gbpa_ctx *ctx, int ne, int D, int Q, const double *B,
                         const double *qd, double *y);

// Deterministic CSR scatter E -> L: y[i] = sum_j +-xE[indices[j]]; with
// ess_mask, y[i] = xc[i] on constrained dofs (ConstrainedOperator DIAG_ONE).
template <typename T>
int launch_csr_scatter(gbpa_ctx *ctx, int ndofs, const int *offsets,
                       const int *indices, const T *xE, T *y,
                       const unsigned char *ess_mask, const T *xc, bool add,
                       bool abs_values);

// out[i] = gather_map[i], or GBPA_GATHER_SKIP where the slot's dof is masked.
int launch_masked_gather_map(gbpa_ctx *ctx, int64_t n, const int *gather_map,
                             const unsigned char *mask, int *out);

// nbz chosen for (kind, precision, D, Q): tuned table or default.
int elements_per_block(int kind, int precision, int D, int Q);
// Thread layout of the gather-fused apply for (kind, precision, D, Q):
// GBPA_LAYOUT_SLAB2D (default) or GBPA_LAYOUT_3D, with *nbz the 3D kernel's
// elements per block.
int apply_layout(int kind, int precision, int D, int Q, int *nbz);
// FP32 block diffusion apply: GBPA_LAYOUT_TC or GBPA_LAYOUT_SLAB2D for (D, Q, nrhs)
int block_apply_layout(int D, int Q, int nrhs);

// Vector mass with a matrix coefficient (vdim 3): block-major qdata
// (Q^3, NE, 9), y_E += sum over the coupled blocks (gbpa_vector_coupled.cu).
int vector_mass_apply_matrix(gbpa_ctx *ctx, int ne, int d1d, int q1d, const double *B, const double *D,
                             const double *x, double *y);

// Deterministic two-level dot product into a device scalar (double).
template <typename T>
int launch_dot(gbpa_ctx *ctx, int64_t n, const T *x, const T *y,
               double *d_result);
} // namespace gbpa
