// Allocation-free L-vector diffusion apply.
//
// Some callers of this library cannot allocate device memory. For example, an
// application that hands every byte of the GPU to its own pool allocator (as an
// MFEM build with a host-managed device memory pool does), or code on a path
// that must not trigger the implicit device synchronisation cudaMalloc/cudaFree
// can cause. gbpa_operator_mult needs an E-vector of scratch, which the
// operator allocates with cudaMalloc. This entry point computes the same
// y = R^T A_e R x for FP64 diffusion, but its E-vector lives in the fixed
// file-scope device array below, so the call itself allocates nothing.
//
// Limits and sharing rules:
//  - ne * d1d^3 must not exceed GBPA_NOALLOC_MAX_EVEC doubles (16 MiB of
//    scratch, held by every GPU that loads the library until the process
//    exits); larger problems are rejected with GBPA_ERR_UNSUPPORTED.
//  - All calls share the one array. Calls whose work overlaps on the GPU (two
//    streams at once, or two host threads) race on it; serialise them.
//  - The array keeps the last call's contents. Nothing needs clearing: the
//    element kernel overwrites every scratch entry it later reads.
//  - The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress and keeps it for the life of the process; make that
//    first call before any stream capture. The kept address belongs to the
//    device's primary context: do not call this entry point again after a
//    cudaDeviceReset (or any other teardown of that context).
#include "gbpa_dispatch.cuh"
#include <mutex>

static __device__ __align__(256) double g_noalloc_evec[GBPA_NOALLOC_MAX_EVEC];

namespace
{
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_evec_ptr[kMaxDevices] = {};
}

extern "C" int gbpa_diffusion_mult_noalloc(void *stream, int ne, int ndofs, int d1d, int q1d,
                                           int symm, const double *B, const double *G,
                                           const double *qdata, const int *gather_map,
                                           const int *offsets, const int *indices,
                                           const double *x, double *y)
{
   if (ne < 0 || ndofs < 0 || d1d < 1 || q1d < 1) { return GBPA_ERR_INVALID_ARGUMENT; }
   // sizes beyond the kernels' range: the same code as the rest of the ABI
   if (d1d > GBPA_MAX_1D || q1d > GBPA_MAX_1D) { return GBPA_ERR_UNSUPPORTED; }
   const long long nE = (long long)ne * d1d * d1d * d1d;
   if (nE > GBPA_NOALLOC_MAX_EVEC)
   {
      fprintf(stderr, "gbpa_diffusion_mult_noalloc: ne*d1d^3 = %lld exceeds the fixed scratch of "
              "%d doubles; use gbpa_operator_mult\n", nE, GBPA_NOALLOC_MAX_EVEC);
      return GBPA_ERR_UNSUPPORTED;
   }
   if (ndofs == 0) { return GBPA_SUCCESS; }
   if (!x || !y || !offsets || (ne > 0 && (!B || !G || !qdata || !gather_map || !indices)))
   {
      return GBPA_ERR_INVALID_ARGUMENT;
   }
   int dev = 0;
   int rc = gbpa::check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
   if (rc) { return rc; }
   if (dev < 0 || dev >= kMaxDevices) { return GBPA_ERR_UNSUPPORTED; }
   double *evec = nullptr;
   {
      std::lock_guard<std::mutex> lock(g_mu);
      if (!g_evec_ptr[dev])
      {
         void *p = nullptr;
         rc = gbpa::check_cuda(cudaGetSymbolAddress(&p, g_noalloc_evec), "cudaGetSymbolAddress");
         if (rc) { return rc; }
         g_evec_ptr[dev] = (double *)p;
      }
      evec = g_evec_ptr[dev];
   }
   // a context on the stack: stream and launch bookkeeping only, no memory
   gbpa_ctx c;
   c.device = dev;
   c.stream = (cudaStream_t)stream;
   rc = gbpa::launch_diffusion_apply<double>(&c, ne, symm ? 1 : 0, d1d, q1d, B, G, qdata, x,
                                             gather_map, nullptr, evec, false);
   if (rc) { return rc; }
   return gbpa::launch_csr_scatter<double>(&c, ndofs, offsets, indices, evec, y, nullptr, nullptr,
                                           false, false);
}
