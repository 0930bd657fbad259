// Deterministic CSR row sum of an E-vector: the transpose of the element
// restriction (ElementRestriction::MultTranspose, fem/restriction.cpp:159-201),
// y[i] = sum over j in [offsets[i], offsets[i+1]) of +-xE[k_j] with
// k_j = indices[j] (or -1 - indices[j] for a flipped sign), in row order.
#pragma once
#include <cstdint>

namespace gbpa
{
// The row's index loads are issued together (8 at a time; an H1 dof in 3D
// has at most 8 element slots), then its value loads, so the dependent
// loads overlap instead of taking one round trip per entry. The sum is
// accumulated in row order, so it is bit-identical to the plain loop.
//   stride, lane  xE[k * stride + lane] (interleaved right-hand sides)
//   COH           read xE through L2 (written by other blocks of the launch)
template <typename T, bool COH = false>
__device__ __forceinline__ T csr_row_sum(const int *__restrict__ offsets, const int *__restrict__ indices,
                                         const T *__restrict__ xE, int i, bool use_abs = false,
                                         int stride = 1, int lane = 0)
{
   constexpr int U = 8;
   const int j0 = offsets[i], j1 = offsets[i + 1];
   T v = T(0);
   for (int j = j0; j < j1; j += U)
   {
      int s[U];
#pragma unroll
      for (int u = 0; u < U; ++u) { s[u] = j + u < j1 ? indices[j + u] : 0; }
      T a[U];
#pragma unroll
      for (int u = 0; u < U; ++u)
      {
         a[u] = T(0);
         if (j + u < j1)
         {
            const int k = s[u] >= 0 ? s[u] : -1 - s[u];
            const T *p = xE + (int64_t)k * stride + lane;
            a[u] = COH ? __ldcg(p) : *p;
         }
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
      {
         if (j + u < j1) { v += (s[u] >= 0 || use_abs) ? a[u] : -a[u]; }
      }
   }
   return v;
}

// R interleaved values of one E-vector slot (or one dof), loaded as one
// vector: R * sizeof(T) bytes, aligned to that size.
template <typename T, int R>
struct alignas(sizeof(T) * R) RhsVec
{
   T v[R];
};

// csr_row_sum for all R interleaved right-hand sides of row i at once:
// the row's indices are loaded once, each slot's R values in one vector load,
// and out[r] is summed in row order (bit-identical to csr_row_sum with
// stride R, lane r). U slots are in flight per thread, 128 bytes of values.
template <typename T, int R>
__device__ __forceinline__ void csr_row_sum_rhs(const int *__restrict__ offsets,
                                                const int *__restrict__ indices,
                                                const T *__restrict__ xE, int i, T (&out)[R])
{
   constexpr int UB = 128 / int(sizeof(T) * R);
   constexpr int U = UB < 1 ? 1 : (UB > 8 ? 8 : UB);
   using V = RhsVec<T, R>;
   const V *xv = reinterpret_cast<const V *>(xE);
#pragma unroll
   for (int r = 0; r < R; ++r) { out[r] = T(0); }
   const int j0 = offsets[i], j1 = offsets[i + 1];
   for (int j = j0; j < j1; j += U)
   {
      int s[U];
#pragma unroll
      for (int u = 0; u < U; ++u) { s[u] = j + u < j1 ? indices[j + u] : 0; }
      V a[U];
#pragma unroll
      for (int u = 0; u < U; ++u)
      {
         if (j + u < j1) { a[u] = xv[s[u] >= 0 ? s[u] : -1 - s[u]]; }
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
      {
         if (j + u < j1)
         {
#pragma unroll
            for (int r = 0; r < R; ++r) { out[r] += s[u] >= 0 ? a[u].v[r] : -a[u].v[r]; }
         }
      }
   }
}
} // namespace gbpa
