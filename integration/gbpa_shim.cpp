// libgbpa behind MFEM's partial-assembly bilinear form (see gbpa_shim.hpp).
//
// Host-memory MFEM (built without CUDA, Device("cpu") or Device("omp")): the
// operator is created with gbpa_operator_create_host from the host arrays and
// applied with gbpa_operator_mult_host on the host Vectors; the library moves
// the data and runs restriction, apply and transpose on the GPU. With
// MFEM_USE_CUDA the device pointers of MFEM's Memory go to
// gbpa_operator_create / gbpa_operator_mult directly, on the legacy default
// stream MFEM's kernels use (that build is not made on this pool; the host
// path is the one the tests run).
#include "gbpa_shim.hpp"

#include "mfem.hpp"
#include "gbpa.h"

#include <cstdlib>
#include <mutex>
#include <type_traits>
#include <unordered_map>

namespace mfem
{
namespace gbpa_shim
{
namespace
{
static_assert(std::is_same<real_t, double>::value, "libgbpa's MFEM operator is FP64");

// DiffusionIntegrator keeps its partial-assembly data private
// (fem/bilininteg.hpp: maps, dim, ne, dofs1D, quad1D, pa_data, symmetric).
// Names used in an explicit instantiation are exempt from access checking
// ([temp.explicit]), so each member's pointer is taken there, once, and
// handed out by a friend function -- MFEM's class stays as it is.
template <typename Tag, typename Tag::type M>
struct MemberOf
{
   friend typename Tag::type member(Tag) { return M; }
};
#define GBPA_MEMBER(NAME, TYPE)                                          \
   struct NAME##_tag                                                     \
   {                                                                     \
      typedef TYPE DiffusionIntegrator::*type;                           \
      friend type member(NAME##_tag);                                    \
   };                                                                    \
   template struct MemberOf<NAME##_tag, &DiffusionIntegrator::NAME>;
GBPA_MEMBER(pa_data, Vector)
GBPA_MEMBER(maps, const DofToQuad *)
GBPA_MEMBER(dim, int)
GBPA_MEMBER(ne, int)
GBPA_MEMBER(dofs1D, int)
GBPA_MEMBER(quad1D, int)
GBPA_MEMBER(symmetric, bool)
#undef GBPA_MEMBER

struct DiffusionAccess
{
   static const Vector &PAData(const DiffusionIntegrator &d) { return d.*member(pa_data_tag{}); }
   static const DofToQuad *Maps(const DiffusionIntegrator &d) { return d.*member(maps_tag{}); }
   static int Dim(const DiffusionIntegrator &d) { return d.*member(dim_tag{}); }
   static int NE(const DiffusionIntegrator &d) { return d.*member(ne_tag{}); }
   static int Dofs1D(const DiffusionIntegrator &d) { return d.*member(dofs1D_tag{}); }
   static int Quad1D(const DiffusionIntegrator &d) { return d.*member(quad1D_tag{}); }
   static bool Symmetric(const DiffusionIntegrator &d) { return d.*member(symmetric_tag{}); }
};

struct State
{
   gbpa_operator_t op = nullptr;
   const BilinearFormIntegrator *integ = nullptr;   // the integrator and PA data the
   const real_t *pa = nullptr;                      // operator was built from
   int ndofs = 0;
};

std::mutex g_mu;
std::unordered_map<const void *, State> g_ops;
gbpa_ctx_t g_ctx = nullptr;
long g_forwarded = 0;

void check(int rc, const char *what)
{
   if (rc != GBPA_SUCCESS) { MFEM_ABORT("libgbpa: " << what << " returned " << rc); }
}

bool device_memory()
{
#ifdef MFEM_USE_CUDA
   return Device::Allows(Backend::CUDA_MASK);
#else
   return false;
#endif
}

void release_locked(const void *ext)
{
   auto it = g_ops.find(ext);
   if (it == g_ops.end()) { return; }
   gbpa_operator_destroy(it->second.op);
   g_ops.erase(it);
}
} // namespace

bool Enabled()
{
   static const bool on = [] {
      const char *e = std::getenv("MFEM_GBPA");
      return e && e[0] == '1';
   }();
   return on;
}

void Assemble(const void *ext, BilinearForm &a, const Operator *elem_restrict)
{
   if (!Enabled()) { return; }
   std::lock_guard<std::mutex> lock(g_mu);
   release_locked(ext);
   // forwarded forms: one domain DiffusionIntegrator, no element markers, no
   // boundary or face integrators, scalar H1 on 3D tensor-product elements
   if (a.GetDBFI()->Size() != 1 || a.GetBBFI()->Size() || a.GetFBFI()->Size() || a.GetBFBFI()->Size())
   {
      return;
   }
   if ((*a.GetDBFI_Marker())[0] != nullptr) { return; }
   const auto *di = dynamic_cast<const DiffusionIntegrator *>((*a.GetDBFI())[0]);
   const auto *R = dynamic_cast<const ElementRestriction *>(elem_restrict);
   const FiniteElementSpace *fes = a.FESpace();
   if (!di || !R || fes->GetVDim() != 1 || DiffusionAccess::Dim(*di) != 3) { return; }
   const DofToQuad *maps = DiffusionAccess::Maps(*di);
   const int D = DiffusionAccess::Dofs1D(*di), Q = DiffusionAccess::Quad1D(*di);
   const int ne = DiffusionAccess::NE(*di);
   const bool symm = DiffusionAccess::Symmetric(*di);
   const Vector &pa = DiffusionAccess::PAData(*di);
   if (!maps || maps->mode != DofToQuad::TENSOR || maps->ndof != D || maps->nqpt != Q) { return; }
   if (pa.Size() != (symm ? 6 : 9) * Q * Q * Q * ne || R->GatherMap().Size() != ne * D * D * D) { return; }

   const bool dev = device_memory();
   if (!g_ctx)
   {
      check(gbpa_create(&g_ctx, 0), "gbpa_create");
      // MFEM's device kernels run on the legacy default stream
      if (dev) { check(gbpa_set_stream(g_ctx, reinterpret_cast<void *>(1)), "gbpa_set_stream"); }
   }
   gbpa_operator_desc d{};
   d.kind = GBPA_DIFFUSION;
   d.precision = GBPA_F64;
   d.ne = ne;
   d.ndofs = fes->GetNDofs();
   d.d1d = D;
   d.q1d = Q;
   d.symm = symm ? 1 : 0;
   d.ess = nullptr;
   d.n_ess = 0;
   d.scatter = GBPA_SCATTER_CSR;
   gbpa_operator_t op = nullptr;
   if (dev)
   {
      d.B = maps->B.Read(); d.G = maps->G.Read(); d.qdata = pa.Read();
      d.gather_map = R->GatherMap().Read(); d.offsets = R->Offsets().Read(); d.indices = R->Indices().Read();
      check(gbpa_operator_create(g_ctx, &d, &op), "gbpa_operator_create");
   }
   else
   {
      d.B = maps->B.HostRead(); d.G = maps->G.HostRead(); d.qdata = pa.HostRead();
      d.gather_map = R->GatherMap().HostRead(); d.offsets = R->Offsets().HostRead();
      d.indices = R->Indices().HostRead();
      check(gbpa_operator_create_host(g_ctx, &d, &op), "gbpa_operator_create_host");
   }
   State s;
   s.op = op;
   s.integ = di;
   s.pa = pa.GetData();
   s.ndofs = d.ndofs;
   g_ops[ext] = s;
}

bool Mult(const void *ext, BilinearForm &a, const Vector &x, Vector &y)
{
   if (!Enabled()) { return false; }
   std::lock_guard<std::mutex> lock(g_mu);
   auto it = g_ops.find(ext);
   if (it == g_ops.end()) { return false; }
   const State &s = it->second;
   // the form still holds the integrator and PA data the operator was built from
   if (a.GetDBFI()->Size() != 1 || (*a.GetDBFI())[0] != s.integ) { return false; }
   const auto *di = static_cast<const DiffusionIntegrator *>(s.integ);
   if (DiffusionAccess::PAData(*di).GetData() != s.pa) { return false; }
   if (x.Size() != s.ndofs || y.Size() != s.ndofs) { return false; }
   if (device_memory())
   {
      check(gbpa_operator_mult(s.op, x.Read(), y.Write()), "gbpa_operator_mult");
   }
   else
   {
      check(gbpa_operator_mult_host(s.op, x.HostRead(), y.HostWrite()), "gbpa_operator_mult_host");
   }
   ++g_forwarded;
   return true;
}

void Release(const void *ext)
{
   if (!Enabled()) { return; }
   std::lock_guard<std::mutex> lock(g_mu);
   release_locked(ext);
}

long ForwardedMults()
{
   std::lock_guard<std::mutex> lock(g_mu);
   return g_forwarded;
}

} // namespace gbpa_shim
} // namespace mfem
