// Context, launch plumbing, restriction gather/scatter, reductions and the
// BLAS-1 / Jacobi kernels of the PA path.
//   context            general/device.cpp:191,443-453 (Device("cuda"))
//   restriction        fem/restriction.cpp:26-228
//   dot / reduce       linalg/vector.cpp:1079-1106, general/reducers.hpp:451-594
//   vector add         linalg/vector.cpp:414-600
//   Jacobi setup       linalg/solvers.cpp:401-425
#include "gbpa_csr.cuh"
#include "gbpa_dispatch.cuh"
#include "gbpa_tc.cuh"
#include <cstring>
#include <mutex>
#include <new>
#include <unordered_map>

namespace gbpa
{

int check_cuda(cudaError_t e, const char *what)
{
   if (e == cudaSuccess) { return GBPA_SUCCESS; }
   fprintf(stderr, "gbpa: %s: %s\n", what, cudaGetErrorString(e));
   return e == cudaErrorMemoryAllocation ? GBPA_ERR_OUT_OF_MEMORY : GBPA_ERR_CUDA;
}

void *scratch(gbpa_ctx *ctx, int slot, size_t bytes)
{
   if ((int)ctx->slots.size() <= slot) { ctx->slots.resize(slot + 1); }
   gbpa_ctx::Slot &s = ctx->slots[slot];
   if (s.bytes >= bytes && s.ptr) { return s.ptr; }
   if (s.ptr)
   {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(s.ptr);
      s.ptr = nullptr; s.bytes = 0;
   }
   const size_t want = bytes < 256 ? 256 : bytes;
   if (cudaMalloc(&s.ptr, want) != cudaSuccess)
   {
      cudaGetLastError();
      s.ptr = nullptr;
      return nullptr;
   }
   s.bytes = want;
   return s.ptr;
}

int ensure_smem(const void *kernel, size_t bytes)
{
   static std::mutex mu;
   static std::unordered_map<const void *, size_t> done;
   if (bytes <= 48 * 1024) { return GBPA_SUCCESS; }
   std::lock_guard<std::mutex> lock(mu);
   auto it = done.find(kernel);
   if (it != done.end() && it->second >= bytes) { return GBPA_SUCCESS; }
   const int rc = check_cuda(cudaFuncSetAttribute(
                                kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)bytes), "cudaFuncSetAttribute");
   if (rc == GBPA_SUCCESS) { done[kernel] = bytes; }
   return rc;
}

// Largest block the kernel can launch with (register-limited), cached.
int max_threads_for(const void *kernel)
{
   static std::mutex mu;
   static std::unordered_map<const void *, int> cache;
   std::lock_guard<std::mutex> lock(mu);
   auto it = cache.find(kernel);
   if (it != cache.end()) { return it->second; }
   cudaFuncAttributes a;
   int m = 1024;
   if (cudaFuncGetAttributes(&a, kernel) == cudaSuccess) { m = a.maxThreadsPerBlock; }
   else { cudaGetLastError(); }
   cache[kernel] = m;
   return m;
}

int launch_generic(gbpa_ctx *ctx, const void *kernel, dim3 grid, dim3 block,
                   void **args, size_t smem, const char *what)
{
   if (smem > 227 * 1024) { return GBPA_ERR_UNSUPPORTED; }
   const int threads = (int)(block.x * block.y * block.z);
   if (threads > 1024 || threads > max_threads_for(kernel)) { return GBPA_ERR_UNSUPPORTED; }
   int rc = ensure_smem(kernel, smem);
   if (rc) { return rc; }
   const cudaError_t e = cudaLaunchKernel(kernel, grid, block, args, smem, ctx->stream);
   if (e != cudaSuccess)
   {
      // a refused launch sets the runtime's last-error; clear it so a later,
      // unrelated check does not report it again
      cudaGetLastError();
   }
   rc = check_cuda(e, what);
   ctx->launches++;
   return rc;
}

// ------------------------------------------------ elements per block table
static std::mutex g_nbz_mu;
static std::unordered_map<int, int> g_nbz;
static int nbz_key(int kind, int prec, int D, int Q)
{
   return ((kind * 4 + prec) * 32 + D) * 32 + Q;
}

int elements_per_block(int kind, int prec, int D, int Q)
{
   {
      std::lock_guard<std::mutex> lock(g_nbz_mu);
      auto it = g_nbz.find(nbz_key(kind, prec, D, Q));
      if (it != g_nbz.end()) { return it->second; }
   }
   // default: about 256 threads per block, capped by 1024 threads and by
   // ~100 KB of shared memory so that two blocks fit on an SM
   const int q2 = Q * Q;
   int nbz = 256 / q2;
   if (nbz < 1) { nbz = 1; }
   const size_t w = prec == GBPA_F32 ? 4 : 8;
   const int per = kind == GBPA_DIFFUSION ? 0 : 1;
   (void)per;
   while (nbz > 1)
   {
      const int D3 = D * D * D;
      const int a = D3 > 3 * D * q2 ? D3 : 3 * D * q2;
      const size_t bytes = w * (size_t)nbz * (a + 2 * D * D * Q);
      if (bytes <= 100 * 1024 && nbz * q2 <= 1024) { break; }
      --nbz;
   }
   return nbz;
}

// ------------------------------------------------------------ restriction
__global__ void gather_kernel(int64_t n, int nd, int vdim, int byvdim,
                              int ndofs, const int *__restrict__ gmap,
                              const double *__restrict__ x,
                              double *__restrict__ y, int use_abs)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int g = gmap[i];
      const bool plus = g >= 0 || use_abs;
      const int j = g >= 0 ? g : -1 - g;
      const int64_t ld = i % nd, le = i / nd;
      for (int c = 0; c < vdim; ++c)
      {
         const double v = byvdim ? x[c + (int64_t)vdim * j] : x[j + (int64_t)ndofs * c];
         y[ld + nd * (c + (int64_t)vdim * le)] = plus ? v : -v;
      }
   }
}

__global__ void masked_gather_map_kernel(int64_t n, const int *__restrict__ gmap,
                                         const unsigned char *__restrict__ mask, int *__restrict__ out)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const int g = gmap[i];
      const int j = g >= 0 ? g : -1 - g;
      out[i] = mask[j] ? GBPA_GATHER_SKIP : g;
   }
}

int launch_masked_gather_map(gbpa_ctx *ctx, int64_t n, const int *gather_map, const unsigned char *mask,
                             int *out)
{
   if (n <= 0) { return GBPA_SUCCESS; }
   masked_gather_map_kernel<<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(n, gather_map, mask,
                                                                                        out);
   return last_launch(ctx, "masked_gather_map");
}

template <typename T>
__global__ void csr_scatter_kernel(int ndofs, const int *__restrict__ offsets,
                                   const int *__restrict__ indices,
                                   const T *__restrict__ xE, T *__restrict__ y,
                                   const unsigned char *__restrict__ mask,
                                   const T *__restrict__ xc, int add,
                                   int use_abs)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndofs;
        i += gridDim.x * blockDim.x)
   {
      if (mask && mask[i]) { y[i] = xc[i]; continue; }
      const T v = csr_row_sum<T>(offsets, indices, xE, i, use_abs != 0);
      y[i] = add ? y[i] + v : v;
   }
}

// vdim > 1 scatter (E-vector (nd, vdim, ne))
__global__ void csr_scatter_vdim_kernel(int ndofs, int nd, int vdim, int byvdim,
                                        const int *__restrict__ offsets,
                                        const int *__restrict__ indices,
                                        const double *__restrict__ xE,
                                        double *__restrict__ y, int add,
                                        int use_abs)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndofs;
        i += gridDim.x * blockDim.x)
   {
      for (int c = 0; c < vdim; ++c)
      {
         double v = 0;
         for (int j = offsets[i]; j < offsets[i + 1]; ++j)
         {
            const int s = indices[j];
            const int k = s >= 0 ? s : -1 - s;
            const double a = xE[k % nd + (int64_t)nd * (c + (int64_t)vdim * (k / nd))];
            v += (s >= 0 || use_abs) ? a : -a;
         }
         const int64_t o = byvdim ? c + (int64_t)vdim * i : i + (int64_t)ndofs * c;
         y[o] = add ? y[o] + v : v;
      }
   }
}

template <typename T>
int launch_csr_scatter(gbpa_ctx *ctx, int ndofs, const int *offsets,
                       const int *indices, const T *xE, T *y,
                       const unsigned char *ess_mask, const T *xc, bool add,
                       bool abs_values)
{
   if (ndofs == 0) { return GBPA_SUCCESS; }
   const int block = 256;
   csr_scatter_kernel<T><<<grid_for(ndofs, block), block, 0, ctx->stream>>>(
      ndofs, offsets, indices, xE, y, ess_mask, xc, add ? 1 : 0, abs_values ? 1 : 0);
   return last_launch(ctx, "csr_scatter");
}
template int launch_csr_scatter<double>(gbpa_ctx *, int, const int *, const int *,
                                        const double *, double *, const unsigned char *,
                                        const double *, bool, bool);
template int launch_csr_scatter<float>(gbpa_ctx *, int, const int *, const int *,
                                       const float *, float *, const unsigned char *,
                                       const float *, bool, bool);

// ------------------------------------------------------------- reductions
// Two-level deterministic reduction: each block reduces a fixed strided
// slice (warp shuffles, then one value per warp in shared memory), the last
// block to finish sums the per-block partials in block order.
constexpr int DOT_BLOCK = 512;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) { v += __shfl_down_sync(0xffffffffu, v, o); }
   return v;
}

__device__ double block_sum(double v)
{
   __shared__ double ws[32];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   v = warp_sum(v);
   if (lane == 0) { ws[wid] = v; }
   __syncthreads();
   const int nw = (blockDim.x + 31) >> 5;
   v = (threadIdx.x < nw) ? ws[threadIdx.x] : 0.0;
   if (wid == 0) { v = warp_sum(v); }
   __syncthreads();
   return v;   // valid in thread 0
}

template <typename T>
__global__ void dot_kernel(int64_t n, const T *__restrict__ x,
                           const T *__restrict__ y, double *partials,
                           unsigned int *counter, double *result)
{
   double s = 0.0;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      s += (double)x[i] * (double)y[i];
   }
   s = block_sum(s);
   __shared__ bool last;
   if (threadIdx.x == 0)
   {
      partials[blockIdx.x] = s;
      __threadfence();
      last = atomicInc(counter, gridDim.x - 1) == gridDim.x - 1;
   }
   __syncthreads();
   if (last)
   {
      __threadfence();
      double t = 0.0;
      for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
      {
         t += ((volatile double *)partials)[b];
      }
      t = block_sum(t);
      if (threadIdx.x == 0) { *result = t; }
   }
}

template <typename T>
int launch_dot(gbpa_ctx *ctx, int64_t n, const T *x, const T *y, double *d_result)
{
   const unsigned g = grid_for(n, DOT_BLOCK, 4 * ctx->num_sms);
   dot_kernel<T><<<g, DOT_BLOCK, 0, ctx->stream>>>(n, x, y, ctx->d_partials,
                                                   ctx->d_counter, d_result);
   return last_launch(ctx, "dot");
}
template int launch_dot<double>(gbpa_ctx *, int64_t, const double *, const double *, double *);
template int launch_dot<float>(gbpa_ctx *, int64_t, const float *, const float *, double *);

__global__ void add_kernel(int64_t n, const double *x, double a,
                           const double *y, double *z)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      z[i] = x[i] + a * y[i];
   }
}

__global__ void jacobi_setup_kernel(int64_t n, const double *diag, double damping,
                                    double *dinv, int *flags)
{
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
   {
      const double d = diag[i];
      if (d == 0.0) { atomicOr(flags, GBPA_FLAG_ZERO_DIAGONAL); dinv[i] = 0.0; }
      else { dinv[i] = damping / d; }
   }
}

__global__ void set_at_kernel(int n, const int *idx, double v, double *y)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
   {
      y[idx[i]] = v;
   }
}

} // namespace gbpa

using namespace gbpa;

// ------------------------------------------------------------------- C ABI
extern "C" int gbpa_version(void) { return GBPA_VERSION; }

extern "C" const char *gbpa_error_string(int status)
{
   switch (status)
   {
      case GBPA_SUCCESS: return "success";
      case GBPA_ERR_INVALID_ARGUMENT: return "invalid argument";
      case GBPA_ERR_UNSUPPORTED: return "unsupported size or configuration";
      case GBPA_ERR_CUDA: return "CUDA runtime error";
      case GBPA_ERR_NOT_FINITE: return "non-finite value in solver";
      case GBPA_ERR_ZERO_DIAGONAL: return "zero diagonal entry in Jacobi smoother";
      case GBPA_ERR_NOT_CONVERGED: return "solver did not converge";
      case GBPA_ERR_TIMEOUT: return "device wait timed out";
      case GBPA_ERR_OUT_OF_MEMORY: return "out of device memory";
      case GBPA_ERR_INDEX: return "index map entry out of range";
      default: return "unknown status";
   }
}

extern "C" int gbpa_create(gbpa_ctx_t *out, int device)
{
   if (!out) { return GBPA_ERR_INVALID_ARGUMENT; }
   *out = nullptr;
   int rc = check_cuda(cudaSetDevice(device), "cudaSetDevice");
   if (rc) { return rc; }
   gbpa_ctx *ctx = new (std::nothrow) gbpa_ctx;
   if (!ctx) { return GBPA_ERR_OUT_OF_MEMORY; }
   ctx->device = device;
   cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
   rc = check_cuda(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking),
                   "cudaStreamCreate");
   if (!rc) { rc = check_cuda(cudaMalloc(&ctx->d_flags, 4 * sizeof(int)), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMallocHost(&ctx->h_pinned, 64 * sizeof(double)), "cudaMallocHost"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&ctx->d_scalars, 64 * sizeof(double)), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&ctx->d_counter, 64 * sizeof(unsigned int)), "cudaMalloc"); }
   if (!rc) { rc = check_cuda(cudaMalloc(&ctx->d_partials, 4096 * sizeof(double)), "cudaMalloc"); }
   if (!rc)
   {
      cudaMemset(ctx->d_flags, 0, 4 * sizeof(int));
      cudaMemset(ctx->d_counter, 0, 64 * sizeof(unsigned int));
      rc = check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
   }
   ctx->stream = ctx->own_stream;
   if (rc) { gbpa_destroy(ctx); return rc; }
   *out = ctx;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_destroy(gbpa_ctx_t ctx)
{
   if (!ctx) { return GBPA_SUCCESS; }
   cudaSetDevice(ctx->device);
   if (ctx->stream) { cudaStreamSynchronize(ctx->stream); }
   for (auto &s : ctx->slots) { if (s.ptr) { cudaFree(s.ptr); } }
   if (ctx->d_flags) { cudaFree(ctx->d_flags); }
   if (ctx->h_pinned) { cudaFreeHost(ctx->h_pinned); }
   if (ctx->d_scalars) { cudaFree(ctx->d_scalars); }
   if (ctx->d_counter) { cudaFree(ctx->d_counter); }
   if (ctx->d_partials) { cudaFree(ctx->d_partials); }
   if (ctx->own_stream) { cudaStreamDestroy(ctx->own_stream); }
   if (ctx->capture_stream) { cudaStreamDestroy(ctx->capture_stream); }
   delete ctx;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_set_stream(gbpa_ctx_t ctx, void *stream)
{
   if (!ctx) { return GBPA_ERR_INVALID_ARGUMENT; }
   ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
   return GBPA_SUCCESS;
}

extern "C" void *gbpa_get_stream(gbpa_ctx_t ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" int gbpa_synchronize(gbpa_ctx_t ctx)
{
   if (!ctx) { return GBPA_ERR_INVALID_ARGUMENT; }
   return check_cuda(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
}

extern "C" int gbpa_get_error_flags(gbpa_ctx_t ctx, int *flags)
{
   if (!ctx || !flags) { return GBPA_ERR_INVALID_ARGUMENT; }
   int h = 0;
   int rc = check_cuda(cudaMemcpyAsync(&h, ctx->d_flags, sizeof(int), cudaMemcpyDeviceToHost,
                                       ctx->stream), "cudaMemcpyAsync");
   if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize"); }
   if (!rc) { rc = check_cuda(cudaMemsetAsync(ctx->d_flags, 0, sizeof(int), ctx->stream), "memset"); }
   *flags = h;
   return rc;
}

extern "C" int64_t gbpa_launch_count(gbpa_ctx_t ctx) { return ctx ? ctx->launches : 0; }

extern "C" int gbpa_restriction_build(int ne, int dof, int ndofs, const int *elem_dofs,
                                      const int *dof_map, int *offsets, int *indices,
                                      int *gather_map)
{
   // Host construction with the reference's counting / prefix-sum / fill order
   // (fem/restriction.cpp:72-113), so the maps are identical entry for entry.
   if (ne < 0 || dof <= 0 || ndofs < 0 || !offsets || (ne > 0 && (!elem_dofs || !indices || !gather_map)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   for (int i = 0; i <= ndofs; ++i) { offsets[i] = 0; }
   for (int64_t k = 0; k < (int64_t)ne * dof; ++k)
   {
      const int s = elem_dofs[k];
      const int g = s >= 0 ? s : -1 - s;
      if (g >= ndofs) { return GBPA_ERR_INDEX; }
      ++offsets[g + 1];
   }
   for (int i = 1; i <= ndofs; ++i) { offsets[i] += offsets[i - 1]; }
   for (int e = 0; e < ne; ++e)
   {
      for (int d = 0; d < dof; ++d)
      {
         const int sd = dof_map ? dof_map[d] : 0;
         const int did = dof_map ? (sd >= 0 ? sd : -1 - sd) : d;
         if (did >= dof) { return GBPA_ERR_INDEX; }
         const int sg = elem_dofs[(int64_t)dof * e + did];
         const int g = sg >= 0 ? sg : -1 - sg;
         const int lid = dof * e + d;
         const bool plus = (sg >= 0) == (sd >= 0);
         gather_map[lid] = plus ? g : -1 - g;
         indices[offsets[g]++] = plus ? lid : -1 - lid;
      }
   }
   for (int i = ndofs; i > 0; --i) { offsets[i] = offsets[i - 1]; }
   offsets[0] = 0;
   return GBPA_SUCCESS;
}

// ---------------------------------------------- device-side map construction
// Same maps as the host construction. The CSR fill order within a row must
// follow increasing E-slot order (the reference fills rows while walking
// elements in order), so each row is filled by sorting: count -> scan ->
// scatter the (row, lid) keys with an atomic cursor -> sort each row.
__global__ void rb_count_kernel(int64_t n, const int *elem_dofs, int *counts)
{
   for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
        k += (int64_t)gridDim.x * blockDim.x)
   {
      const int s = elem_dofs[k];
      atomicAdd(counts + (s >= 0 ? s : -1 - s) + 1, 1);
   }
}
__global__ void rb_fill_kernel(int ne, int dof, const int *elem_dofs, const int *dof_map,
                               const int *offsets, int *cursor, int *indices, int *gather_map)
{
   const int64_t n = (int64_t)ne * dof;
   for (int64_t lid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lid < n;
        lid += (int64_t)gridDim.x * blockDim.x)
   {
      const int e = (int)(lid / dof), d = (int)(lid % dof);
      const int sd = dof_map ? dof_map[d] : 0;
      const int did = dof_map ? (sd >= 0 ? sd : -1 - sd) : d;
      const int sg = elem_dofs[(int64_t)dof * e + did];
      const int g = sg >= 0 ? sg : -1 - sg;
      const bool plus = (sg >= 0) == (sd >= 0);
      gather_map[lid] = plus ? g : -1 - g;
      const int pos = offsets[g] + atomicAdd(cursor + g, 1);
      indices[pos] = plus ? (int)lid : (int)(-1 - lid);
   }
}
__global__ void rb_sort_rows_kernel(int ndofs, const int *offsets, int *indices)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndofs; i += gridDim.x * blockDim.x)
   {
      const int j0 = offsets[i], j1 = offsets[i + 1];
      // rows hold at most a few dozen entries: insertion sort on |lid|
      for (int a = j0 + 1; a < j1; ++a)
      {
         const int v = indices[a];
         const int kv = v >= 0 ? v : -1 - v;
         int b = a - 1;
         while (b >= j0)
         {
            const int w = indices[b];
            if ((w >= 0 ? w : -1 - w) <= kv) { break; }
            indices[b + 1] = w;
            --b;
         }
         indices[b + 1] = v;
      }
   }
}
__global__ void rb_scan_kernel(int n, int *a)
{
   // single-block inclusive scan of a[0..n] (n+1 entries), chunked
   __shared__ int carry;
   if (threadIdx.x == 0) { carry = 0; }
   __syncthreads();
   __shared__ int buf[1024];
   for (int base = 0; base <= n; base += 1024)
   {
      const int i = base + threadIdx.x;
      buf[threadIdx.x] = i <= n ? a[i] : 0;
      __syncthreads();
      for (int o = 1; o < 1024; o <<= 1)
      {
         const int v = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
         __syncthreads();
         buf[threadIdx.x] += v;
         __syncthreads();
      }
      if (i <= n) { a[i] = buf[threadIdx.x] + carry; }
      __syncthreads();
      if (threadIdx.x == 1023) { carry += buf[1023]; }
      __syncthreads();
   }
}

extern "C" int gbpa_restriction_build_device(gbpa_ctx_t ctx, int ne, int dof, int ndofs,
                                             const int *elem_dofs, const int *dof_map,
                                             int *offsets, int *indices, int *gather_map)
{
   if (!ctx || ne < 0 || dof <= 0 || ndofs < 0 || !offsets) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (ne == 0)
   {
      return check_cuda(cudaMemsetAsync(offsets, 0, sizeof(int) * (ndofs + 1), ctx->stream), "memset");
   }
   int *cursor = (int *)scratch(ctx, SLOT_RESTRICT, sizeof(int) * (size_t)ndofs);
   if (!cursor) { return GBPA_ERR_OUT_OF_MEMORY; }
   const int64_t n = (int64_t)ne * dof;
   cudaMemsetAsync(offsets, 0, sizeof(int) * (ndofs + 1), ctx->stream);
   cudaMemsetAsync(cursor, 0, sizeof(int) * ndofs, ctx->stream);
   rb_count_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, elem_dofs, offsets);
   int rc = last_launch(ctx, "restriction_count");
   if (rc) { return rc; }
   rb_scan_kernel<<<1, 1024, 0, ctx->stream>>>(ndofs, offsets);
   rc = last_launch(ctx, "restriction_scan");
   if (rc) { return rc; }
   rb_fill_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(ne, dof, elem_dofs, dof_map, offsets,
                                                             cursor, indices, gather_map);
   rc = last_launch(ctx, "restriction_fill");
   if (rc) { return rc; }
   rb_sort_rows_kernel<<<grid_for(ndofs, 256), 256, 0, ctx->stream>>>(ndofs, offsets, indices);
   return last_launch(ctx, "restriction_sort");
}

static int restriction_args_ok(gbpa_ctx_t ctx, int ne, int nd, int vdim, int ndofs)
{
   if (!ctx || ne < 0 || nd <= 0 || ndofs < 0) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (vdim < 1 || vdim > 3) { return GBPA_ERR_UNSUPPORTED; }
   return GBPA_SUCCESS;
}

static int gather_common(gbpa_ctx_t ctx, int ne, int nd, int vdim, int byvdim, int ndofs,
                         const int *gmap, const double *x, double *y, int use_abs)
{
   int rc = restriction_args_ok(ctx, ne, nd, vdim, ndofs);
   if (rc) { return rc; }
   const int64_t n = (int64_t)ne * nd;
   if (n == 0) { return GBPA_SUCCESS; }
   if (!gmap || !x || !y) { return GBPA_ERR_INVALID_ARGUMENT; }
   gather_kernel<<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, nd, vdim, byvdim, ndofs, gmap, x,
                                                            y, use_abs);
   return last_launch(ctx, "restriction_gather");
}

extern "C" int gbpa_restriction_mult(gbpa_ctx_t ctx, int ne, int nd, int vdim, int byvdim,
                                     int ndofs, const int *gather_map, const double *x,
                                     double *y)
{
   return gather_common(ctx, ne, nd, vdim, byvdim, ndofs, gather_map, x, y, 0);
}

extern "C" int gbpa_restriction_abs_mult(gbpa_ctx_t ctx, int ne, int nd, int vdim, int byvdim,
                                         int ndofs, const int *gather_map, const double *x,
                                         double *y)
{
   return gather_common(ctx, ne, nd, vdim, byvdim, ndofs, gather_map, x, y, 1);
}

static int scatter_common(gbpa_ctx_t ctx, int ne, int nd, int vdim, int byvdim, int ndofs,
                          const int *offsets, const int *indices, const double *x,
                          double *y, int add, int use_abs)
{
   int rc = restriction_args_ok(ctx, ne, nd, vdim, ndofs);
   if (rc) { return rc; }
   if (ndofs == 0) { return GBPA_SUCCESS; }
   if (!offsets || !y || (ne > 0 && (!indices || !x))) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (vdim == 1)
   {
      return launch_csr_scatter<double>(ctx, ndofs, offsets, indices, x, y, nullptr, nullptr,
                                        add != 0, use_abs != 0);
   }
   csr_scatter_vdim_kernel<<<grid_for(ndofs, 256), 256, 0, ctx->stream>>>(
      ndofs, nd, vdim, byvdim, offsets, indices, x, y, add, use_abs);
   return last_launch(ctx, "restriction_scatter_vdim");
}

extern "C" int gbpa_restriction_mult_transpose(gbpa_ctx_t ctx, int ne, int nd, int vdim,
                                               int byvdim, int ndofs, const int *offsets,
                                               const int *indices, const double *x,
                                               double *y, int add)
{
   return scatter_common(ctx, ne, nd, vdim, byvdim, ndofs, offsets, indices, x, y, add, 0);
}

extern "C" int gbpa_restriction_abs_mult_transpose(gbpa_ctx_t ctx, int ne, int nd, int vdim,
                                                   int byvdim, int ndofs, const int *offsets,
                                                   const int *indices, const double *x,
                                                   double *y)
{
   return scatter_common(ctx, ne, nd, vdim, byvdim, ndofs, offsets, indices, x, y, 0, 1);
}

extern "C" int gbpa_vec_dot(gbpa_ctx_t ctx, int64_t n, const double *x, const double *y,
                            double *result)
{
   if (!ctx || !result || n < 0 || (n > 0 && (!x || !y))) { return GBPA_ERR_INVALID_ARGUMENT; }
   int rc = launch_dot<double>(ctx, n, x, y, ctx->d_scalars);
   if (rc) { return rc; }
   rc = check_cuda(cudaMemcpyAsync(ctx->h_pinned, ctx->d_scalars, sizeof(double),
                                   cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
   if (!rc) { rc = check_cuda(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize"); }
   *result = ctx->h_pinned[0];
   return rc;
}

extern "C" int gbpa_vec_add(gbpa_ctx_t ctx, int64_t n, const double *x, double a,
                            const double *y, double *z)
{
   if (!ctx || n < 0 || (n > 0 && (!x || !y || !z))) { return GBPA_ERR_INVALID_ARGUMENT; }
   if (n == 0) { return GBPA_SUCCESS; }
   add_kernel<<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(n, x, a, y, z);
   return last_launch(ctx, "vec_add");
}

extern "C" int gbpa_jacobi_setup(gbpa_ctx_t ctx, int64_t n, const double *diag, const int *ess,
                                 int n_ess, double damping, double *dinv)
{
   if (!ctx || n < 0 || n_ess < 0 || (n > 0 && (!diag || !dinv)) || (n_ess > 0 && !ess))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (n == 0) { return GBPA_SUCCESS; }
   int flags = 0;
   int rc = gbpa_get_error_flags(ctx, &flags);   // clear stale flags
   if (rc) { return rc; }
   jacobi_setup_kernel<<<grid_for(n, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(
      n, diag, damping, dinv, ctx->d_flags);
   rc = last_launch(ctx, "jacobi_setup");
   if (rc) { return rc; }
   if (n_ess > 0)
   {
      set_at_kernel<<<grid_for(n_ess, 256), 256, 0, ctx->stream>>>(n_ess, ess, damping, dinv);
      rc = last_launch(ctx, "jacobi_setup_ess");
      if (rc) { return rc; }
   }
   rc = gbpa_get_error_flags(ctx, &flags);
   if (rc) { return rc; }
   return (flags & GBPA_FLAG_ZERO_DIAGONAL) ? GBPA_ERR_ZERO_DIAGONAL : GBPA_SUCCESS;
}

extern "C" int gbpa_set_elements_per_block(int kind, int precision, int d1d, int q1d, int nbz)
{
   if (kind < 0 || kind > 1 || precision < 0 || precision > 2 || d1d < 1 || q1d < 1 ||
       d1d > GBPA_MAX_1D || q1d > GBPA_MAX_1D || nbz < 0 || nbz * q1d * q1d > 1024)
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   std::lock_guard<std::mutex> lock(g_nbz_mu);
   if (nbz == 0) { g_nbz.erase(nbz_key(kind, precision, d1d, q1d)); }
   else { g_nbz[nbz_key(kind, precision, d1d, q1d)] = nbz; }
   return GBPA_SUCCESS;
}

extern "C" int gbpa_get_elements_per_block(int kind, int precision, int d1d, int q1d)
{
   if (kind < 0 || kind > 1 || precision < 0 || precision > 2) { return GBPA_ERR_INVALID_ARGUMENT; }
   return elements_per_block(kind, precision, d1d, q1d);
}

// ------------------------------------------------------ apply layout table
// key -> (layout, nbz of the 3D layout); absent = the 2D slab
static std::unordered_map<int, std::pair<int, int>> g_layout;

int gbpa::apply_layout(int kind, int precision, int D, int Q, int *nbz)
{
   std::lock_guard<std::mutex> lock(g_nbz_mu);
   auto it = g_layout.find(nbz_key(kind, precision, D, Q));
   if (it == g_layout.end()) { return GBPA_LAYOUT_SLAB2D; }
   if (nbz) { *nbz = it->second.second; }
   return it->second.first;
}

extern "C" int gbpa_set_apply_layout(int kind, int precision, int d1d, int q1d, int layout, int nbz)
{
   if (kind < 0 || kind > 1 || precision < 0 || precision > 2 || d1d < 1 || q1d < 1 ||
       d1d > GBPA_MAX_1D || q1d > GBPA_MAX_1D ||
       (layout != GBPA_LAYOUT_SLAB2D && layout != GBPA_LAYOUT_3D && layout != GBPA_LAYOUT_TC) ||
       (layout == GBPA_LAYOUT_3D && (nbz < 1 || nbz * q1d * q1d * q1d > 1024 || nbz * q1d > 64)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (layout == GBPA_LAYOUT_TC &&
       (kind != GBPA_DIFFUSION || precision != GBPA_F32 || !gbpa::tc::supported(d1d, q1d)))
   {
      return GBPA_ERR_UNSUPPORTED;
   }
   std::lock_guard<std::mutex> lock(g_nbz_mu);
   if (layout == GBPA_LAYOUT_SLAB2D) { g_layout.erase(nbz_key(kind, precision, d1d, q1d)); }
   else { g_layout[nbz_key(kind, precision, d1d, q1d)] = {layout, layout == GBPA_LAYOUT_3D ? nbz : 0}; }
   return GBPA_SUCCESS;
}

// FP32 block diffusion apply, per (D, Q, nrhs): the tensor-core kernel where
// one exists, unless set to the CUDA-core block kernel
static std::unordered_map<int, int> g_block_layout;

static int block_key(int D, int Q, int nrhs) { return (D * 64 + Q) * 64 + nrhs; }

int gbpa::block_apply_layout(int D, int Q, int nrhs)
{
   if (!gbpa::tc::block_supported(D, Q, nrhs)) { return GBPA_LAYOUT_SLAB2D; }
   std::lock_guard<std::mutex> lock(g_nbz_mu);
   auto it = g_block_layout.find(block_key(D, Q, nrhs));
   return it == g_block_layout.end() ? GBPA_LAYOUT_TC : it->second;
}

extern "C" int gbpa_set_block_apply_layout(int d1d, int q1d, int nrhs, int layout)
{
   if (d1d < 1 || q1d < 1 || d1d > GBPA_MAX_1D || q1d > GBPA_MAX_1D || nrhs < 1 ||
       (layout != GBPA_LAYOUT_SLAB2D && layout != GBPA_LAYOUT_TC))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   if (layout == GBPA_LAYOUT_TC && !gbpa::tc::block_supported(d1d, q1d, nrhs)) { return GBPA_ERR_UNSUPPORTED; }
   std::lock_guard<std::mutex> lock(g_nbz_mu);
   g_block_layout[block_key(d1d, q1d, nrhs)] = layout;
   return GBPA_SUCCESS;
}

extern "C" int gbpa_get_block_apply_layout(int d1d, int q1d, int nrhs)
{
   if (d1d < 1 || q1d < 1 || d1d > GBPA_MAX_1D || q1d > GBPA_MAX_1D || nrhs < 1) { return GBPA_ERR_INVALID_ARGUMENT; }
   return gbpa::block_apply_layout(d1d, q1d, nrhs);
}

extern "C" int gbpa_get_apply_layout(int kind, int precision, int d1d, int q1d, int *nbz)
{
   if (kind < 0 || kind > 1 || precision < 0 || precision > 2) { return GBPA_ERR_INVALID_ARGUMENT; }
   int n = 0;
   const int layout = gbpa::apply_layout(kind, precision, d1d, q1d, &n);
   if (nbz) { *nbz = layout == GBPA_LAYOUT_3D ? n : elements_per_block(kind, precision, d1d, q1d); }
   return layout;
}
