// Launchers for the apply kernels, templated on the arithmetic. Each
// gbpa_apply_<arith>_<kind>.cu instantiates them for one arithmetic so the
// translation units compile in parallel.
//   GEN    largest D1D/Q1D of the generic (runtime-size) kernel
//   PLAIN  also instantiate the E-vector-input kernels (no gather); the
//          double-float arithmetic is only used by the fused L-vector
//          operator, which always gathers
#pragma once
#include "gbpa_apply_kernels.cuh"
#include "gbpa_dispatch.cuh"
#include <algorithm>
#include <type_traits>

namespace gbpa
{

template <typename AR, bool GATHER, int GEN>
static const void *diffusion_kernel_for(int D, int Q)
{
#define GBPA_CASE(d, q) \
   if (D == d && Q == q) { return (const void *)diffusion_apply_kernel<AR, d, q, GATHER>; }
   GBPA_DQ_LIST(GBPA_CASE)
#undef GBPA_CASE
   return (const void *)diffusion_apply_kernel<AR, 0, 0, GATHER, GEN, GEN>;
}

template <typename AR, bool GATHER, int GEN>
static const void *mass_kernel_for(int D, int Q)
{
#define GBPA_CASE(d, q) \
   if (D == d && Q == q) { return (const void *)mass_apply_kernel<AR, d, q, GATHER>; }
   GBPA_DQ_LIST(GBPA_CASE)
#undef GBPA_CASE
   return (const void *)mass_apply_kernel<AR, 0, 0, GATHER, GEN, GEN>;
}

template <typename AR>
static const void *diffusion_3d_kernel_for(int D, int Q)
{
#define GBPA_CASE(d, q) \
   if (D == d && Q == q) { return (const void *)diffusion_apply_3d_kernel<AR, d, q>; }
   GBPA_DQ3_LIST(GBPA_CASE)
#undef GBPA_CASE
   return nullptr;
}

// Gather-fused diffusion apply in the 3D layout; GBPA_ERR_UNSUPPORTED when no
// compile-time kernel exists for (D, Q).
template <typename AR>
int launch_diffusion_3d_ar(gbpa_ctx *ctx, int ne, int symm, int D, int Q,
                           const typename AR::In *B, const typename AR::In *G,
                           const typename AR::Qd *qd, const typename AR::In *x,
                           const int *gather_map, const unsigned char *ess_mask,
                           typename AR::In *y, int mode, const int *skip, int nbz)
{
   const void *k = diffusion_3d_kernel_for<AR>(D, Q);
   if (!k || !gather_map) { return GBPA_ERR_UNSUPPORTED; }
   const int q3 = Q * Q * Q;
   // blockDim.z = Q * nbz is limited to 64, the block to the kernel's thread limit
   nbz = std::max(1, std::min(nbz, std::min(max_threads_for(k) / q3, 64 / Q)));
   if (q3 > max_threads_for(k)) { return GBPA_ERR_UNSUPPORTED; }
   const int b1 = std::max(D * D * D, 3 * D * Q * Q), b2 = std::max(2 * D * D * Q, 3 * q3);
   const size_t smem = sizeof(typename AR::V) * (2 * Q * D + (size_t)nbz * (b1 + b2));
   void *args[] = {&ne, &symm, (void *)&B, (void *)&G, (void *)&qd, (void *)&x,
                   (void *)&gather_map, (void *)&ess_mask, &y, &mode, (void *)&skip};
   return launch_generic(ctx, k, dim3((ne + nbz - 1) / nbz), dim3(Q, Q, Q * nbz), args, smem,
                         "diffusion_apply_3d");
}

template <typename AR>
static const void *mass_3d_kernel_for(int D, int Q)
{
#define GBPA_CASE(d, q) \
   if (D == d && Q == q) { return (const void *)mass_apply_3d_kernel<AR, d, q>; }
   GBPA_DQ3_LIST(GBPA_CASE)
#undef GBPA_CASE
   return nullptr;
}

// Gather-fused mass apply in the 3D layout; GBPA_ERR_UNSUPPORTED when (D, Q)
// has no 3D kernel.
template <typename AR>
int launch_mass_3d_ar(gbpa_ctx *ctx, int ne, int D, int Q, const typename AR::In *B,
                      const typename AR::Qd *qd, const typename AR::In *x, const int *gather_map,
                      const unsigned char *ess_mask, typename AR::In *y, int mode, const int *skip, int nbz)
{
   const void *k = mass_3d_kernel_for<AR>(D, Q);
   if (!k || !gather_map) { return GBPA_ERR_UNSUPPORTED; }
   const int q3 = Q * Q * Q;
   if (q3 > max_threads_for(k)) { return GBPA_ERR_UNSUPPORTED; }
   nbz = std::max(1, std::min(nbz, std::min(max_threads_for(k) / q3, 64 / Q)));
   const int b1 = std::max(D * D * D, D * Q * Q), b2 = std::max(D * D * Q, q3);
   const size_t smem = sizeof(typename AR::V) * (Q * D + (size_t)nbz * (b1 + b2));
   void *args[] = {&ne, (void *)&B, (void *)&qd, (void *)&x, (void *)&gather_map, (void *)&ess_mask, &y,
                   &mode, (void *)&skip};
   return launch_generic(ctx, k, dim3((ne + nbz - 1) / nbz), dim3(Q, Q, Q * nbz), args, smem, "mass_apply_3d");
}

template <typename AR, int GEN = GBPA_MAX_1D, bool PLAIN = true>
int launch_diffusion_ar(gbpa_ctx *ctx, int prec, int ne, int symm, int D, int Q,
                        const typename AR::In *B, const typename AR::In *G,
                        const typename AR::Qd *qd, const typename AR::In *x,
                        const int *gather_map, const unsigned char *ess_mask,
                        typename AR::In *y, int accumulate, const int *skip)
{
   if (ne == 0) { return GBPA_SUCCESS; }
   if (D > GEN || Q > GEN) { return GBPA_ERR_UNSUPPORTED; }
   int nbz3 = 0;
   if (gather_map && apply_layout(GBPA_DIFFUSION, prec, D, Q, &nbz3) == GBPA_LAYOUT_3D)
   {
      int rc;
      if constexpr (std::is_same<AR, ArF64>::value)
      {
         rc = launch_diffusion_3d_f64(ctx, ne, symm, D, Q, B, G, qd, x, gather_map, ess_mask, y, accumulate,
                                      skip, nbz3);
      }
      else if constexpr (std::is_same<AR, ArF32>::value)
      {
         rc = launch_diffusion_3d_f32(ctx, ne, symm, D, Q, B, G, qd, x, gather_map, ess_mask, y, accumulate,
                                      skip, nbz3);
      }
      else
      {
         rc = launch_diffusion_3d_x2(ctx, ne, symm, D, Q, B, G, qd, x, gather_map, ess_mask, y, accumulate,
                                     skip, nbz3);
      }
      if (rc != GBPA_ERR_UNSUPPORTED) { return rc; }
   }
   const void *k = nullptr;
   if (gather_map) { k = diffusion_kernel_for<AR, true, GEN>(D, Q); }
   else if constexpr (PLAIN) { k = diffusion_kernel_for<AR, false, GEN>(D, Q); }
   else { return GBPA_ERR_UNSUPPORTED; }
   // tuned elements per block, clamped to the kernel's register-limited size
   const int nbz = std::max(1, std::min(elements_per_block(GBPA_DIFFUSION, prec, D, Q),
                                        max_threads_for(k) / (Q * Q)));
   size_t smem = sizeof(typename AR::V) * (2 * Q * D + (size_t)nbz * diff_smem_per_elem(D, Q));
   // TMA staging of the block's qdata when the arithmetic asks for it; the
   // kernel copies the enclosing 16-byte-aligned range, so only the array base
   // has to be 16-byte aligned (tile + 32 bytes of rounding slack + barrier)
   const size_t qbytes = sizeof(typename AR::Qd) * (symm ? 6 : 9) * (size_t)Q * Q * Q;
   int tma = (AR::kTmaQd && ((uintptr_t)qd % 16 == 0)) ? 1 : 0;
   if (tma)
   {
      const size_t with = ((smem + 15) & ~size_t(15)) + nbz * qbytes + 48;
      if (with <= 200 * 1024) { smem = with; }
      else { tma = 0; }
   }
   int acc = accumulate;
   void *args[] = {&ne, &symm, &D, &Q, (void *)&B, (void *)&G, (void *)&qd,
                   (void *)&x, (void *)&gather_map, (void *)&ess_mask, &y, &acc,
                   (void *)&skip, &tma};
   return launch_generic(ctx, k, dim3((ne + nbz - 1) / nbz), dim3(Q, Q, nbz),
                         args, smem, "diffusion_apply");
}

// Block (multi right-hand side) diffusion apply: compile-time kernels for
// Q = D + 1, the generic kernel otherwise.
template <typename AR>
static const void *diffusion_block_kernel_for(int D, int Q, int nrhs)
{
   // 8 right-hand sides (the combined form's count): strides known at compile time
#define GBPA_CASE(d) \
   if (D == d && Q == d + 1) \
   { \
      return nrhs == 8 ? (const void *)diffusion_apply_block_kernel<AR, d, d + 1, 8> \
                       : (const void *)diffusion_apply_block_kernel<AR, d, d + 1>; \
   }
   GBPA_CASE(2) GBPA_CASE(3) GBPA_CASE(4) GBPA_CASE(5) GBPA_CASE(6) GBPA_CASE(7) GBPA_CASE(8)
#undef GBPA_CASE
   return (const void *)diffusion_apply_block_kernel<AR, 0, 0>;
}

template <typename AR>
int launch_diffusion_block_ar(gbpa_ctx *ctx, int ne, int nrhs, int symm, int D, int Q,
                              const typename AR::In *B, const typename AR::In *G,
                              const typename AR::Qd *qd, const typename AR::In *x,
                              const int *gather_map, const unsigned char *ess_mask,
                              typename AR::In *y, const int *skip)
{
   if (ne == 0) { return GBPA_SUCCESS; }
   const void *k = diffusion_block_kernel_for<AR>(D, Q, nrhs);
   const int max_thr = max_threads_for(k);   // register-limited block size
   if (Q * Q > max_thr) { return GBPA_ERR_UNSUPPORTED; }
   const int prec = sizeof(typename AR::V) == 4 ? GBPA_F32 : GBPA_F64;
   const int nbz = std::max(1, std::min(elements_per_block(GBPA_DIFFUSION, prec, D, Q), max_thr / (Q * Q)));
   size_t smem = sizeof(typename AR::V) * (2 * Q * D + (size_t)nbz * diff_smem_per_elem(D, Q));
   // qdata staged once per block for all right-hand sides (16-byte aligned base)
   const size_t qbytes = sizeof(typename AR::Qd) * (symm ? 6 : 9) * (size_t)Q * Q * Q;
   int tma = ((uintptr_t)qd % 16 == 0) ? 1 : 0;
   if (tma)
   {
      const size_t with = ((smem + 15) & ~size_t(15)) + nbz * qbytes + 48;
      if (with <= 200 * 1024) { smem = with; }
      else { tma = 0; }
   }
   void *args[] = {&ne, &nrhs, &symm, &D, &Q, (void *)&B, (void *)&G, (void *)&qd, (void *)&x,
                   (void *)&gather_map, (void *)&ess_mask, &y, (void *)&skip, &tma};
   return launch_generic(ctx, k, dim3((ne + nbz - 1) / nbz), dim3(Q, Q, nbz), args, smem,
                         "diffusion_apply_block");
}

template <typename AR, int GEN = GBPA_MAX_1D, bool PLAIN = true>
int launch_mass_ar(gbpa_ctx *ctx, int prec, int ne, int D, int Q,
                   const typename AR::In *B, const typename AR::Qd *qd,
                   const typename AR::In *x, const int *gather_map,
                   const unsigned char *ess_mask, typename AR::In *y,
                   int accumulate, const int *skip, int qdiv = 1)
{
   if (ne == 0) { return GBPA_SUCCESS; }
   if (D > GEN || Q > GEN) { return GBPA_ERR_UNSUPPORTED; }
   int nbz3 = 0;
   if (gather_map && qdiv == 1 && apply_layout(GBPA_MASS, prec, D, Q, &nbz3) == GBPA_LAYOUT_3D)
   {
      int rc;
      if constexpr (std::is_same<AR, ArF64>::value)
      {
         rc = launch_mass_3d_f64(ctx, ne, D, Q, B, qd, x, gather_map, ess_mask, y, accumulate, skip, nbz3);
      }
      else if constexpr (std::is_same<AR, ArF32>::value)
      {
         rc = launch_mass_3d_f32(ctx, ne, D, Q, B, qd, x, gather_map, ess_mask, y, accumulate, skip, nbz3);
      }
      else
      {
         rc = launch_mass_3d_x2(ctx, ne, D, Q, B, qd, x, gather_map, ess_mask, y, accumulate, skip, nbz3);
      }
      if (rc != GBPA_ERR_UNSUPPORTED) { return rc; }
   }
   const void *k = nullptr;
   if (gather_map) { k = mass_kernel_for<AR, true, GEN>(D, Q); }
   else if constexpr (PLAIN) { k = mass_kernel_for<AR, false, GEN>(D, Q); }
   else { return GBPA_ERR_UNSUPPORTED; }
   const int nbz = std::max(1, std::min(elements_per_block(GBPA_MASS, prec, D, Q),
                                        max_threads_for(k) / (Q * Q)));
   const size_t smem = sizeof(typename AR::V) * (Q * D + (size_t)nbz * mass_smem_per_elem(D, Q));
   int acc = accumulate;
   void *args[] = {&ne, &D, &Q, (void *)&B, (void *)&qd, (void *)&x,
                   (void *)&gather_map, (void *)&ess_mask, &y, &acc, (void *)&skip, &qdiv};
   return launch_generic(ctx, k, dim3((ne + nbz - 1) / nbz), dim3(Q, Q, nbz),
                         args, smem, "mass_apply");
}

} // namespace gbpa
