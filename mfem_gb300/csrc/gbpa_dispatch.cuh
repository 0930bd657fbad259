// Compile-time (D, Q) specialisations and the runtime lookup that replaces
// the reference's kernel dispatch table (fem/kernel_dispatch.hpp:139-153):
// specialised instances for the orders the benchmarks use, the generic
// runtime-size instance otherwise.
#pragma once
#include "gbpa_internal.cuh"

// (D, Q) pairs with compile-time kernels: Q = D (p+1 points), Q = D+1 (p+2,
// the default diffusion/mass rule), and the two extra rules the reference
// also specialises (fem/integ/bilininteg_diffusion_kernels.cpp:81-82).
#define GBPA_DQ_LIST(X)                                                      \
   X(2, 2) X(2, 3) X(3, 3) X(3, 4) X(4, 4) X(4, 5) X(5, 5) X(5, 6) X(6, 6)    \
   X(6, 7) X(7, 7) X(7, 8) X(8, 8) X(8, 9) X(9, 9) X(9, 10) X(4, 6) X(5, 8)

// (D, Q) pairs with a compile-time 3D-layout diffusion kernel: all of the
// above (Q^3 <= 1000 threads per element).
#define GBPA_DQ3_LIST(X) GBPA_DQ_LIST(X)

namespace gbpa
{
// Raise the dynamic shared-memory limit of a kernel once per size class.
int ensure_smem(const void *kernel, size_t bytes);
int launch_generic(gbpa_ctx *ctx, const void *kernel, dim3 grid, dim3 block,
                   void **args, size_t smem, const char *what);
// Largest block size the kernel can be launched with (register-limited).
int max_threads_for(const void *kernel);
} // namespace gbpa
