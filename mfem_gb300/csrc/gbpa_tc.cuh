// Tensor-core (tcgen05) FP32 diffusion apply: tables and launcher
// (gbpa_apply_tc.cu).
#pragma once
#include "gbpa_internal.cuh"

namespace gbpa
{
namespace tc
{
// The Kronecker matrix of one (D, Q) pair, split into fp16 limbs and laid out
// per chunk for the tensor cores (one copy serves both GEMMs), in device
// memory; R is the largest absolute row sum of the matrix (the bound behind
// the per-element output scale).
struct Tables
{
   unsigned char *fwd = nullptr;
   double R = 0.0;
   int D = 0, Q = 0;
};
// (D, Q) pairs with a tensor-core kernel.
bool supported(int D, int Q);
// B, G: host (Q, D) column-major tables in FP64.
int build_tables(int D, int Q, const double *B, const double *G, Tables *t);
void free_tables(Tables *t);
// Per-element power-of-two scale of the pointwise output (one float each).
int launch_qscale(gbpa_ctx *ctx, int ne, int Q, const float *qd, float R, float *qscale);
// The qdata (Q^3, 6, NE) re-laid per tile of 128 elements for the kernel's
// coalesced loads (transposed_qdata_size floats).
int64_t transposed_qdata_size(int D, int Q, int ne);
int launch_transpose_qdata(gbpa_ctx *ctx, int ne, int D, int Q, const float *qd, float *qT);
// y = A_e R x with the gather fused (mode as for the other element kernels:
// 0 E-vector out, 1 accumulate, GBPA_OUT_ATOMIC L-vector). qd: the
// transposed qdata (launch_transpose_qdata) of symmetric FP32 qdata. skip: optional device flag; nonzero skips the launch
// (a solver that has converged inside a captured graph).
int launch_diffusion_f32(gbpa_ctx *ctx, int ne, int D, int Q, const Tables &t, const float *qd,
                         const float *qscale, const float *x, const int *gmap, const unsigned char *mask,
                         float *y, int mode, const int *skip = nullptr);

// Block form (gbpa_apply_tc_block.cu): nrhs right-hand sides stored
// interleaved (x[j nrhs + r]), block E-vector out (y[(e D^3 + i) nrhs + r]);
// a tile is 128 / nrhs elements times nrhs vectors.
bool block_supported(int D, int Q, int nrhs);
int build_block_tables(int D, int Q, const double *B, const double *G, Tables *t);
// The qdata re-laid per tile of 128 / nrhs elements (block_qdata_size floats).
int64_t block_qdata_size(int D, int Q, int nrhs, int ne);
int launch_block_transpose_qdata(gbpa_ctx *ctx, int ne, int D, int Q, int nrhs, const float *qd, float *qT);
int launch_diffusion_block_f32(gbpa_ctx *ctx, int ne, int D, int Q, int nrhs, const Tables &t, const float *qT,
                               const float *qscale, const float *x, const int *gmap, const unsigned char *mask,
                               float *y, const int *skip = nullptr);
} // namespace tc
} // namespace gbpa
