// Grouped element apply of the batched PCG: one launch covers every element
// batch of the active problems that share an order (D, Q), so each order runs
// its compile-time kernel (the same slab code as the single-operator apply)
// at full occupancy, however small the individual problems are. A block whose
// problem has converged returns at once.
#pragma once
#include "gbpa_apply_kernels.cuh"
#include "gbpa_batched.cuh"
#include "gbpa_dispatch.cuh"
#include <algorithm>
#include <type_traits>

namespace gbpa
{
constexpr int BATCH_GEN = 10;   // largest D1D / Q1D of the grouped apply

template <typename AR, int TD, int TQ, int MAXD, int MAXQ>
__global__ void batched_apply_kernel(const BBatch *__restrict__ batches, const BProb *__restrict__ probs,
                                     const BScal *__restrict__ scal, int tma)
{
   const BBatch bt = batches[blockIdx.x];
   if (scal[bt.prob].done) { return; }   // uniform over the block
   const BProb &pr = probs[bt.prob];
   const typename AR::Qd *qd;
   // the split (hi, lo) copy for the double-float arithmetic, the FP64 qdata
   // otherwise (selected by type: both element types are 8 bytes)
   if constexpr (std::is_same<typename AR::Qd, float2>::value) { qd = pr.qd2; }
   else { qd = pr.qd; }
   diffusion_apply_slab<AR, TD, TQ, true, MAXD, MAXQ>(pr.ne, bt.e0, bt.count, 1, pr.D, pr.Q, pr.B, pr.G, qd,
                                                      pr.d, pr.gmap, nullptr, pr.yE, 0, tma);
}

// The same in the 3D thread layout (block (Q, Q, Q * nbz)), for the orders
// whose single-operator apply the autotuner put in that layout.
template <typename AR, int D, int Q>
__global__ void __launch_bounds__(1024, 2)
batched_apply_3d_kernel(const BBatch *__restrict__ batches, const BProb *__restrict__ probs,
                        const BScal *__restrict__ scal)
{
   const BBatch bt = batches[blockIdx.x];
   if (scal[bt.prob].done) { return; }   // uniform over the block
   const BProb &pr = probs[bt.prob];
   const typename AR::Qd *qd;
   if constexpr (std::is_same<typename AR::Qd, float2>::value) { qd = pr.qd2; }
   else { qd = pr.qd; }
   diffusion_3d_block<AR, D, Q>(bt.e0, bt.count, 1, pr.B, pr.G, qd, pr.d, pr.gmap, nullptr, pr.yE, 0);
}

template <typename AR>
static const void *batched_apply_3d_kernel_for(int D, int Q)
{
#define GBPA_CASE(d) \
   if (D == d && Q == d + 1) { return (const void *)batched_apply_3d_kernel<AR, d, d + 1>; }
   GBPA_CASE(2) GBPA_CASE(3) GBPA_CASE(4) GBPA_CASE(5) GBPA_CASE(6) GBPA_CASE(7)
#undef GBPA_CASE
   return nullptr;
}

// Elements per block of the 3D grouped apply for (precision, D, Q), or 0 when
// that order runs in the 2D slab.
template <typename AR>
static int batched_apply_3d_nbz(int prec, int D, int Q)
{
   int n3 = 0;
   if (apply_layout(GBPA_DIFFUSION, prec, D, Q, &n3) != GBPA_LAYOUT_3D) { return 0; }
   const void *k = batched_apply_3d_kernel_for<AR>(D, Q);
   if (!k) { return 0; }
   const int q3 = Q * Q * Q;
   if (q3 > max_threads_for(k)) { return 0; }
   return std::max(1, std::min(n3, std::min(max_threads_for(k) / q3, 64 / Q)));
}

// Compile-time kernels for p = 1..6 with the default rule Q = D + 1, the
// generic runtime-size kernel otherwise.
template <typename AR>
static const void *batched_apply_kernel_for(int D, int Q)
{
#define GBPA_CASE(d) \
   if (D == d && Q == d + 1) { return (const void *)batched_apply_kernel<AR, d, d + 1, d, d + 1>; }
   GBPA_CASE(2) GBPA_CASE(3) GBPA_CASE(4) GBPA_CASE(5) GBPA_CASE(6) GBPA_CASE(7)
#undef GBPA_CASE
   return (const void *)batched_apply_kernel<AR, 0, 0, BATCH_GEN, BATCH_GEN>;
}

template <typename AR>
int batched_apply_nbz_ar(int prec, int D, int Q)
{
   if (D < 1 || Q < 1 || D > BATCH_GEN || Q > BATCH_GEN) { return 0; }
   const int n3 = batched_apply_3d_nbz<AR>(prec, D, Q);
   if (n3 > 0) { return n3; }
   const int m = max_threads_for(batched_apply_kernel_for<AR>(D, Q)) / (Q * Q);
   if (m < 1) { return 0; }
   return std::max(1, std::min(elements_per_block(GBPA_DIFFUSION, prec, D, Q), m));
}

template <typename AR>
int launch_batched_apply_ar(gbpa_ctx *ctx, int D, int Q, int nbz, const BBatch *batches, int nbatch,
                            const BProb *probs, const BScal *scal)
{
   if (nbatch == 0) { return GBPA_SUCCESS; }
   const int prec = std::is_same<typename AR::Qd, float2>::value ? GBPA_F64X2 : GBPA_F64;
   if (batched_apply_3d_nbz<AR>(prec, D, Q) > 0)
   {
      // the batches were cut with the 3D layout's elements per block (nbz)
      const void *k3 = batched_apply_3d_kernel_for<AR>(D, Q);
      const int b1 = std::max(D * D * D, 3 * D * Q * Q), b2 = std::max(2 * D * D * Q, 3 * Q * Q * Q);
      const size_t smem3 = sizeof(typename AR::V) * (2 * Q * D + (size_t)nbz * (b1 + b2));
      void *args3[] = {(void *)&batches, (void *)&probs, (void *)&scal};
      return launch_generic(ctx, k3, dim3(nbatch), dim3(Q, Q, Q * nbz), args3, smem3, "batched_apply_3d");
   }
   const void *k = batched_apply_kernel_for<AR>(D, Q);
   const size_t smem = sizeof(typename AR::V) * (2 * Q * D + (size_t)nbz * diff_smem_per_elem(D, Q));
   // the batched arithmetics (FP64, double-float) read qdata straight from
   // global memory: no TMA staging
   int tma = 0;
   void *args[] = {(void *)&batches, (void *)&probs, (void *)&scal, &tma};
   return launch_generic(ctx, k, dim3(nbatch), dim3(Q, Q, nbz), args, smem, "batched_apply");
}
} // namespace gbpa
