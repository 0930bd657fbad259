// Golden-vector generator. Runs the UNMODIFIED reference MFEM (serial CPU
// build made by oracle/ref/Makefile) through its public partial-assembly API
// and writes every intermediate of the PA H1 path as .npy files:
//   ElementRestriction maps      fem/restriction.cpp:26-114
//   DofToQuad B/G tables         fem/fe/fe_base.cpp:2697-2741
//   Jacobians / determinants     mesh/mesh.cpp:15445-15500
//   PADiffusionSetup3D qdata     fem/integ/bilininteg_diffusion_kernels.cpp:262-386
//   AddMultPA / AssembleDiagonal fem/integ/bilininteg_{diffusion,mass}_pa.cpp
//   BilinearForm::Mult (PA)      fem/bilinearform_ext.cpp:487-564
//   PCG + OperatorJacobiSmoother linalg/solvers.cpp:331-452,869-1050
//   DomainLFIntegrator (device)  fem/linearform_ext.cpp:20-68
//   VectorDiffusionIntegrator PA fem/integ/bilininteg_vecdiffusion_pa.cpp
//   p-multigrid (transfer, Chebyshev smoother, V-cycle): run_pmg below
// Usage: golden_driver <outdir>   (one subdirectory per case)
#include "mfem.hpp"
#include "fem/integ/bilininteg_diffusion_kernels.hpp"
#include <cstdio>
#include <cstdint>
#include <cmath>
#include <string>
#include <vector>
#include <sys/stat.h>

using namespace mfem;

// ---------------------------------------------------------------- npy writer
static void write_npy(const std::string &path, const char *descr,
                      const std::vector<long> &shape, const void *data,
                      size_t elem_size)
{
   std::string hdr = "{'descr': '";
   hdr += descr;
   hdr += "', 'fortran_order': False, 'shape': (";
   size_t n = 1;
   for (size_t i = 0; i < shape.size(); i++)
   {
      hdr += std::to_string(shape[i]);
      hdr += (shape.size() == 1 || i + 1 < shape.size()) ? ", " : "";
      n *= shape[i];
   }
   hdr += "), }";
   size_t total = 10 + hdr.size() + 1;
   size_t pad = (64 - total % 64) % 64;
   hdr += std::string(pad, ' ');
   hdr += "\n";
   FILE *f = fopen(path.c_str(), "wb");
   if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(1); }
   const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
   fwrite(magic, 1, 8, f);
   uint16_t hl = (uint16_t)hdr.size();
   fwrite(&hl, 2, 1, f);
   fwrite(hdr.data(), 1, hdr.size(), f);
   if (n) { fwrite(data, elem_size, n, f); }
   fclose(f);
}
static void save(const std::string &dir, const char *name, const Vector &v)
{
   write_npy(dir + "/" + name + ".npy", "<f8", {(long)v.Size()},
             v.HostRead(), 8);
}
static void save(const std::string &dir, const char *name,
                 const Array<real_t> &v)
{
   write_npy(dir + "/" + name + ".npy", "<f8", {(long)v.Size()},
             v.HostRead(), 8);
}
static void save(const std::string &dir, const char *name, const Array<int> &v)
{
   write_npy(dir + "/" + name + ".npy", "<i4", {(long)v.Size()},
             v.HostRead(), 4);
}
static void save_ints(const std::string &dir, const char *name,
                      const std::vector<int> &v)
{
   write_npy(dir + "/" + name + ".npy", "<i4", {(long)v.size()}, v.data(), 4);
}
static void save_dbls(const std::string &dir, const char *name,
                      const std::vector<double> &v)
{
   write_npy(dir + "/" + name + ".npy", "<f8", {(long)v.size()}, v.data(), 8);
}

// ------------------------------------------- synthetic inputs (shared recipe)
// splitmix64 stream: the same generator is used by the GPU library's mesh
// builder, so jittered vertices and coefficient modes are identical.
static uint64_t splitmix64(uint64_t &s)
{
   uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
   z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
   z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
   return z ^ (z >> 31);
}
static double u01(uint64_t &s) { return (splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

struct Modes { int k[16][3]; double phi[16]; };
static Modes make_modes(uint64_t seed)
{
   Modes m; uint64_t s = seed;
   for (int i = 0; i < 16; i++)
   {
      for (int d = 0; d < 3; d++) { m.k[i][d] = (int)(u01(s) * 9.0) - 4; }
      m.phi[i] = 2.0 * M_PI * u01(s);
   }
   return m;
}
static Modes g_modes;
static double kappa_fn(const Vector &x)
{
   double g = 0.0;
   for (int i = 0; i < 16; i++)
   {
      const double a = 2.0 * M_PI * (g_modes.k[i][0] * x(0) + g_modes.k[i][1] * x(1) +
                                     g_modes.k[i][2] * x(2)) + g_modes.phi[i];
      g += 0.5 * cos(a);
   }
   return exp(g);
}
static void vec_kappa_fn(const Vector &x, Vector &v)
{
   v.SetSize(3);
   const double k = kappa_fn(x);
   v(0) = k; v(1) = 1.0 + 0.5 * x(0); v(2) = 2.0 - x(1) * x(2);
}
static void sym_mat_fn(const Vector &x, DenseMatrix &M)
{
   M.SetSize(3);
   const double k = kappa_fn(x);
   M(0,0) = 2.0 + k;  M(0,1) = 0.3 * x(2); M(0,2) = 0.1;
   M(1,0) = M(0,1);   M(1,1) = 3.0 - x(0); M(1,2) = -0.2 * x(1);
   M(2,0) = M(0,2);   M(2,1) = M(1,2);     M(2,2) = 2.5 + x(1);
}
static void sym_mat_fn_s(const Vector &x, DenseSymmetricMatrix &M)
{
   DenseMatrix F; sym_mat_fn(x, F);
   M.SetSize(3);
   for (int i = 0; i < 3; i++) for (int j = i; j < 3; j++) { M(i, j) = F(i, j); }
}
static void nonsym_mat_fn(const Vector &x, DenseMatrix &M)
{
   sym_mat_fn(x, M);
   M(0,1) += 0.25; M(2,0) -= 0.15 * x(0); M(1,2) += 0.05;
}
static void curve_map(const Vector &x, Vector &y)
{
   y = x;
   const double s = 0.05 * sin(2 * M_PI * x(0)) * sin(2 * M_PI * x(1)) *
                    sin(2 * M_PI * x(2));
   for (int d = 0; d < 3; d++) { y(d) = x(d) + s; }
}

static void jitter_vertices(Mesh &mesh, int n, double amp, uint64_t seed)
{
   // Interior vertices move by U(-amp*h, amp*h) in each coordinate; three
   // draws are consumed per vertex (in vertex order) whether it moves or not.
   const double h = 1.0 / n;
   uint64_t s = seed;
   for (int v = 0; v < mesh.GetNV(); v++)
   {
      real_t *c = mesh.GetVertex(v);
      bool interior = true;
      for (int d = 0; d < 3; d++)
      {
         if (!(c[d] > 1e-12 && c[d] < 1.0 - 1e-12)) { interior = false; }
      }
      for (int d = 0; d < 3; d++)
      {
         const double r = u01(s);
         if (interior) { c[d] += (2.0 * r - 1.0) * amp * h; }
      }
   }
}

enum CoeffKind { C_ONE = 0, C_FN = 1, C_VEC = 2, C_SYM = 3, C_NONSYM = 4, C_CONST = 5 };

struct Case
{
   const char *name;
   int n, p, q;       // elements per side, order, quadrature points per dim
   double jitter;     // vertex jitter amplitude in units of h
   int coeff;         // CoeffKind
   bool curved;       // order-3 curved geometry (x + 0.05 sin sin sin)
   bool solve;        // cfg1-style Dirichlet Poisson + Jacobi-PCG
};

static void run_case(const Case &c, const std::string &root)
{
   const std::string dir = root + "/" + c.name;
   mkdir(dir.c_str(), 0755);
   Mesh mesh = Mesh::MakeCartesian3D(c.n, c.n, c.n, Element::HEXAHEDRON,
                                     1.0, 1.0, 1.0, true);
   if (c.jitter > 0) { jitter_vertices(mesh, c.n, c.jitter, 1); }
   {
      std::vector<double> vtx(3 * mesh.GetNV());
      for (int v = 0; v < mesh.GetNV(); v++)
      {
         for (int d = 0; d < 3; d++) { vtx[3*v+d] = mesh.GetVertex(v)[d]; }
      }
      save_dbls(dir, "vertices", vtx);
      std::vector<int> ev(8 * mesh.GetNE());
      for (int e = 0; e < mesh.GetNE(); e++)
      {
         Array<int> vv; mesh.GetElementVertices(e, vv);
         for (int k = 0; k < 8; k++) { ev[8*e+k] = vv[k]; }
      }
      save_ints(dir, "elem_vertices", ev);
   }
   if (c.curved)
   {
      mesh.SetCurvature(3, false, 3, Ordering::byVDIM);
      mesh.Transform(curve_map);
   }
   mesh.EnsureNodes();

   H1_FECollection fec(c.p, 3);
   FiniteElementSpace fes(&mesh, &fec);
   const int ndofs = fes.GetNDofs();
   const int ne = mesh.GetNE();
   const int p = c.p, q = c.q;
   const IntegrationRule &ir = IntRules.Get(Geometry::CUBE, 2 * q - 1);
   MFEM_VERIFY(ir.GetNPoints() == q * q * q, "rule size");

   // --- restriction maps (a1)
   const ElementRestriction *R = dynamic_cast<const ElementRestriction*>(
      fes.GetElementRestriction(ElementDofOrdering::LEXICOGRAPHIC));
   MFEM_VERIFY(R, "expected ElementRestriction");
   save(dir, "gather_map", R->GatherMap());
   save(dir, "offsets", R->Offsets());
   save(dir, "indices", R->Indices());
   {
      const Table &e2d = fes.GetElementToDofTable();
      std::vector<int> j(e2d.GetJ(), e2d.GetJ() + e2d.Size_of_connections());
      save_ints(dir, "elem_dofs", j);
      auto el_t = dynamic_cast<const TensorBasisElement*>(fes.GetTypicalFE());
      save(dir, "dof_map", el_t->GetDofMap());
   }

   // --- basis tables and geometry (a5-a7)
   const FiniteElement &el = *fes.GetTypicalFE();
   const DofToQuad &maps = el.GetDofToQuad(ir, DofToQuad::TENSOR);
   save(dir, "B", maps.B); save(dir, "G", maps.G);
   save(dir, "Bt", maps.Bt); save(dir, "Gt", maps.Gt);
   save(dir, "W", ir.GetWeights());
   {
      // nodal (geometry) space: E-vector of nodes and its tables
      const FiniteElementSpace *nfes = mesh.GetNodalFESpace();
      const GridFunction *nodes = mesh.GetNodes();
      const Operator *nR = nfes->GetElementRestriction(ElementDofOrdering::LEXICOGRAPHIC);
      Vector nodesE(nR->Height());
      nR->Mult(*nodes, nodesE);
      save(dir, "nodesE", nodesE);
      const DofToQuad &nmaps = nfes->GetTypicalFE()->GetDofToQuad(ir, DofToQuad::TENSOR);
      save(dir, "Bg", nmaps.B); save(dir, "Gg", nmaps.G);
   }
   const GeometricFactors *geom = mesh.GetGeometricFactors(
      ir, GeometricFactors::JACOBIANS | GeometricFactors::DETERMINANTS);
   if (!c.solve) { save(dir, "J", geom->J); }
   save(dir, "detJ", geom->detJ);

   // --- coefficients
   g_modes = make_modes(3);
   ConstantCoefficient one(1.0), twelve(12.34);
   FunctionCoefficient kfn(kappa_fn);
   VectorFunctionCoefficient kvec(3, vec_kappa_fn);
   SymmetricMatrixFunctionCoefficient ksym(3, sym_mat_fn_s);
   MatrixFunctionCoefficient knon(3, nonsym_mat_fn);
   QuadratureSpace qs(mesh, ir);
   CoefficientVector cv(qs, CoefficientStorage::COMPRESSED);
   DiffusionIntegrator *dint = nullptr;
   Coefficient *mass_coeff = nullptr;
   switch (c.coeff)
   {
      case C_ONE: cv.SetConstant(1.0); dint = new DiffusionIntegrator(&ir); mass_coeff = &one; break;
      case C_CONST: cv.SetConstant(12.34); dint = new DiffusionIntegrator(twelve, &ir); mass_coeff = &twelve; break;
      case C_FN: cv.Project(kfn); dint = new DiffusionIntegrator(kfn, &ir); mass_coeff = &kfn; break;
      case C_VEC: cv.Project(kvec); dint = new DiffusionIntegrator(kvec, &ir); mass_coeff = &kfn; break;
      case C_SYM: cv.ProjectTranspose(ksym); dint = new DiffusionIntegrator(ksym, &ir); mass_coeff = &kfn; break;
      case C_NONSYM: cv.ProjectTranspose(knon); dint = new DiffusionIntegrator(knon, &ir); mass_coeff = &kfn; break;
   }
   save(dir, "coeff", cv);
   std::vector<int> meta = {ne, ndofs, p + 1, q, cv.GetVDim(), c.coeff, c.n};
   save_ints(dir, "meta", meta);

   // --- qdata through the reference's own setup kernel (a8)
   const int coeff_dim = cv.GetVDim();
   const bool symm = coeff_dim != 9;
   Vector qd((symm ? 6 : 9) * q * q * q * ne);
   if (!c.solve)
   {
      internal::PADiffusionSetup(3, 3, p + 1, q, coeff_dim, ne, ir.GetWeights(),
                                 geom->J, cv, qd);
      save(dir, "qdata_diff", qd);
   }
   {
      // mass qdata: v(q,e) = W(q) * coeff * detJ (fem/integ/bilininteg_mass_pa.cpp:73-89)
      CoefficientVector mc(*mass_coeff, qs, CoefficientStorage::COMPRESSED);
      save(dir, "coeff_mass", mc);
      const int NQ = q * q * q;
      Vector mq(NQ * ne);
      const bool cc = mc.Size() == 1;
      for (int e = 0; e < ne; e++)
         for (int k = 0; k < NQ; k++)
            mq(k + NQ * e) = ir.GetWeights()[k] * (cc ? mc(0) : mc(k + NQ * e)) *
                             geom->detJ(k + NQ * e);
      if (!c.solve) { save(dir, "qdata_mass", mq); }
   }

   // --- operator applications through BilinearForm (PA)
   Vector x(ndofs);
   {
      uint64_t s = 2;
      for (int i = 0; i < ndofs; i++) { x(i) = 2.0 * u01(s) - 1.0; }
   }
   save(dir, "x", x);
   Vector dof_xyz(3 * ndofs);
   for (int d = 0; d < 3; d++)
   {
      GridFunction gx(&fes);
      FunctionCoefficient fc([d](const Vector &pt) { return pt(d); });
      gx.ProjectCoefficient(fc);
      for (int i = 0; i < ndofs; i++) { dof_xyz(3 * i + d) = gx(i); }
   }
   save(dir, "dof_xyz", dof_xyz);

   BilinearForm a(&fes);
   a.SetAssemblyLevel(AssemblyLevel::PARTIAL);
   a.AddDomainIntegrator(dint);
   a.Assemble();
   Vector y(ndofs); a.Mult(x, y); save(dir, "y_diff", y);
   Vector diag(ndofs); a.AssembleDiagonal(diag); save(dir, "diag_diff", diag);
   {
      Vector xE(R->Height()), yE(R->Height());
      R->Mult(x, xE); yE = 0.0;
      dint->AddMultPA(xE, yE);
      if (!c.solve) { save(dir, "xE", xE); save(dir, "yE_diff", yE); }
      Vector dE(R->Height()); dE = 0.0; dint->AssembleDiagonalPA(dE);
      if (!c.solve) { save(dir, "diagE_diff", dE); }
   }
   if (!c.solve && std::string(c.name) == "jit3_p3_fn")
   {
      // domain-integrator element markers (AddDomainIntegrator(integ, marker):
      // AddMultWithMarkers and the marked diagonal) on a copy of the mesh
      // whose element e has attribute 1 + e % 3, marker {1, 0, 1}; same dofs
      Mesh mm(mesh, true);
      std::vector<int> attr(ne);
      for (int e = 0; e < ne; e++) { attr[e] = 1 + e % 3; mm.SetAttribute(e, attr[e]); }
      mm.SetAttributes();
      FiniteElementSpace fm(&mm, &fec);
      Array<int> marker(3);
      marker[0] = 1; marker[1] = 0; marker[2] = 1;
      BilinearForm am(&fm);
      am.SetAssemblyLevel(AssemblyLevel::PARTIAL);
      am.AddDomainIntegrator(new DiffusionIntegrator(kfn, &ir), marker);
      am.Assemble();
      Vector ymk(ndofs); am.Mult(x, ymk); save(dir, "y_diff_markers", ymk);
      Vector dmk(ndofs); am.AssembleDiagonal(dmk); save(dir, "diag_diff_markers", dmk);
      save_ints(dir, "elem_attr", attr);
      save(dir, "markers", marker);
   }

   BilinearForm m(&fes);
   m.SetAssemblyLevel(AssemblyLevel::PARTIAL);
   MassIntegrator *mint = new MassIntegrator(*mass_coeff, &ir);
   m.AddDomainIntegrator(mint);
   m.Assemble();
   Vector ym(ndofs); m.Mult(x, ym); save(dir, "y_mass", ym);
   Vector dm(ndofs); m.AssembleDiagonal(dm); save(dir, "diag_mass", dm);
   if (!c.solve)
   {
      Vector xE(R->Height()), yE(R->Height());
      R->Mult(x, xE); yE = 0.0;
      mint->AddMultPA(xE, yE); save(dir, "yE_mass", yE);
   }

   if (!c.solve && c.coeff == C_NONSYM)
   {
      // VectorDiffusionIntegrator / VectorMassIntegrator PA with the case's
      // (nonsymmetric) matrix coefficient on the vdim = 3 space (byNODES):
      // components coupled through the coefficient
      // (fem/integ/bilininteg_vecdiffusion_pa.cpp:64-68,119-130,213-272;
      // fem/integ/bilininteg_vecmass_pa.cpp:73-78,119-160), and the
      // coefficient as both setups project it (ProjectTranspose)
      FiniteElementSpace vfes(&mesh, &fec, 3);
      const Operator *vR = vfes.GetElementRestriction(ElementDofOrdering::LEXICOGRAPHIC);
      Vector vx(vfes.GetVSize());
      uint64_t sv = 5;
      for (int i = 0; i < vx.Size(); i++) { vx(i) = 2.0 * u01(sv) - 1.0; }
      Vector vxE(vR->Height());
      vR->Mult(vx, vxE);
      VectorDiffusionIntegrator *vdi = new VectorDiffusionIntegrator(knon);
      vdi->SetIntRule(&ir);
      BilinearForm va(&vfes);
      va.SetAssemblyLevel(AssemblyLevel::PARTIAL);
      va.AddDomainIntegrator(vdi);
      va.Assemble();
      Vector vy(vfes.GetVSize());
      va.Mult(vx, vy);
      Vector vyE(vR->Height());
      vyE = 0.0;
      vdi->AddMultPA(vxE, vyE);
      save(dir, "vec_x", vx);
      save(dir, "vec_xE", vxE);
      save(dir, "vmat_y", vy);
      save(dir, "vmat_yE", vyE);
      VectorMassIntegrator *vmi = new VectorMassIntegrator(knon);
      vmi->SetIntRule(&ir);
      BilinearForm vm(&vfes);
      vm.SetAssemblyLevel(AssemblyLevel::PARTIAL);
      vm.AddDomainIntegrator(vmi);
      vm.Assemble();
      Vector vmy(vfes.GetVSize());
      vm.Mult(vx, vmy);
      Vector vmyE(vR->Height());
      vmyE = 0.0;
      vmi->AddMultPA(vxE, vmyE);
      save(dir, "vmatmass_y", vmy);
      save(dir, "vmatmass_yE", vmyE);
      CoefficientVector mc(qs, CoefficientStorage::FULL);
      mc.ProjectTranspose(knon);
      save(dir, "vmat_coeff", mc);
   }

   if (!c.solve && (c.coeff == C_FN || c.coeff == C_VEC))
   {
      // VectorDiffusionIntegrator PA on the vdim = 3 space (byNODES) with the
      // case's scalar or vector coefficient and rule
      // (fem/integ/bilininteg_vecdiffusion_pa.cpp:68-276, apply
      // fem/integ/bilininteg_vecdiffusion_pa.hpp:96-163)
      FiniteElementSpace vfes(&mesh, &fec, 3);
      VectorDiffusionIntegrator *vdi = c.coeff == C_FN ? new VectorDiffusionIntegrator(kfn, &ir)
                                                        : new VectorDiffusionIntegrator(kvec);
      if (c.coeff == C_VEC) { vdi->SetIntRule(&ir); }
      const Operator *vR = vfes.GetElementRestriction(ElementDofOrdering::LEXICOGRAPHIC);
      Vector vx(vfes.GetVSize());
      uint64_t sv = 5;
      for (int i = 0; i < vx.Size(); i++) { vx(i) = 2.0 * u01(sv) - 1.0; }
      BilinearForm va(&vfes);
      va.SetAssemblyLevel(AssemblyLevel::PARTIAL);
      va.AddDomainIntegrator(vdi);
      va.Assemble();
      Vector vy(vfes.GetVSize());
      va.Mult(vx, vy);
      Vector vxE(vR->Height()), vyE(vR->Height());
      vR->Mult(vx, vxE);
      vyE = 0.0;
      vdi->AddMultPA(vxE, vyE);
      save(dir, "vec_x", vx);
      save(dir, "vec_y", vy);
      save(dir, "vec_xE", vxE);
      save(dir, "vec_yE", vyE);
      // VectorMassIntegrator PA with the same coefficient and the case's rule
      // (fem/integ/bilininteg_vecmass_pa.cpp:21-210)
      VectorMassIntegrator *vmi = c.coeff == C_FN ? new VectorMassIntegrator(kfn, &ir)
                                                   : new VectorMassIntegrator(kvec);
      if (c.coeff == C_VEC) { vmi->SetIntRule(&ir); }
      BilinearForm vm(&vfes);
      vm.SetAssemblyLevel(AssemblyLevel::PARTIAL);
      vm.AddDomainIntegrator(vmi);
      vm.Assemble();
      Vector vmy(vfes.GetVSize());
      vm.Mult(vx, vmy);
      Vector vmyE(vR->Height());
      vmyE = 0.0;
      vmi->AddMultPA(vxE, vmyE);
      save(dir, "vmass_y", vmy);
      save(dir, "vmass_yE", vmyE);
      if (c.coeff == C_FN)
      {
         CoefficientVector vc(kfn, qs, CoefficientStorage::FULL);
         save(dir, "vmass_coeff", vc);
      }
      else
      {
         CoefficientVector vc(kvec, qs, CoefficientStorage::FULL);
         save(dir, "vmass_coeff", vc);
      }
   }

   if (!c.solve)
   {
      // DomainLFIntegrator(kappa) through the device-style assembly
      // (LinearForm::UseFastAssembly -> LinearFormExtension::Assemble,
      // fem/linearform_ext.cpp:20-68, DLFEvalAssemble3D,
      // fem/integ/lininteg_domain_kernels.hpp:164-...) with its default rule
      // of order 2p (p + 1 Gauss points), and the inputs at that rule
      const IntegrationRule &lir = IntRules.Get(Geometry::CUBE, 2 * p);
      const int lq = p + 1;
      MFEM_VERIFY(lir.GetNPoints() == lq * lq * lq, "lf rule size");
      LinearForm lf(&fes);
      lf.AddDomainIntegrator(new DomainLFIntegrator(kfn));
      lf.UseFastAssembly(true);
      lf.Assemble();
      save(dir, "lf_fn", lf);
      LinearForm lf2(&fes);
      lf2.AddDomainIntegrator(new DomainLFIntegrator(kfn));
      lf2.Assemble();
      save(dir, "lf_fn_host", lf2);
      const DofToQuad &lmaps = el.GetDofToQuad(lir, DofToQuad::TENSOR);
      save(dir, "lf_B", lmaps.B);
      save(dir, "lf_W", lir.GetWeights());
      const GeometricFactors *lgeom = mesh.GetGeometricFactors(lir, GeometricFactors::DETERMINANTS);
      save(dir, "lf_detJ", lgeom->detJ);
      QuadratureSpace lqs(mesh, lir);
      CoefficientVector lcv(kfn, lqs, CoefficientStorage::COMPRESSED);
      save(dir, "lf_coeff", lcv);
   }

   if (c.solve)
   {
      // cfg1: f = 1, homogeneous Dirichlet on the whole boundary, PCG + Jacobi
      Array<int> ess_tdof_list, ess_bdr(mesh.bdr_attributes.Max());
      ess_bdr = 1;
      fes.GetEssentialTrueDofs(ess_bdr, ess_tdof_list);
      save(dir, "ess_tdofs", ess_tdof_list);
      LinearForm b(&fes);
      b.AddDomainIntegrator(new DomainLFIntegrator(one));
      b.Assemble();
      save(dir, "b", b);
      GridFunction xs(&fes); xs = 0.0;
      OperatorPtr A; Vector X, Bv;
      a.FormLinearSystem(ess_tdof_list, xs, b, A, X, Bv);
      save(dir, "B_rhs", Bv);
      Vector Ax(ndofs); A->Mult(x, Ax); save(dir, "Ax_constrained", Ax);
      OperatorJacobiSmoother M(a, ess_tdof_list);
      Vector Mx(ndofs); M.Mult(x, Mx); save(dir, "Mx_jacobi", Mx);
      CGSolver cg;
      cg.SetRelTol(1e-12); cg.SetAbsTol(0.0); cg.SetMaxIter(500);
      cg.SetPrintLevel(0);
      cg.SetOperator(*A); cg.SetPreconditioner(M);
      cg.Mult(Bv, X);
      a.RecoverFEMSolution(X, b, xs);
      save(dir, "X", X);
      std::vector<double> info = {(double)cg.GetNumIterations(), cg.GetFinalNorm(),
                                  (double)cg.GetConverged()};
      save_dbls(dir, "cg_info", info);
      printf("%s: PCG iterations %d final norm %.6e\n", c.name,
             cg.GetNumIterations(), cg.GetFinalNorm());
   }
   printf("%s: ne=%d ndofs=%d D=%d Q=%d coeff_dim=%d\n", c.name, ne, ndofs,
          p + 1, q, coeff_dim);
}

// p-multigrid case (examples/ex26.cpp's structure with a variable kappa):
// orders 1, 2, 4 on one jittered mesh; TransferOperator between the orders
// (TensorProductPRefinementTransferOperator, fem/transfer.cpp:2620-2990);
// OperatorChebyshevSmoother of order 2 on levels 1, 2 (linalg/solvers.cpp:
// 455-660, its eigenvalue estimate from PowerMethod, linalg/operator.cpp:
// 886-942); CGSolver to 1e-2 (max 200) on level 0; Multigrid V(1,1)
// (fem/multigrid.cpp:106-239) as the preconditioner of CGSolver to 1e-10.
static void run_pmg(const std::string &root)
{
   const std::string dir = root + "/pmg4_p124";
   mkdir(dir.c_str(), 0755);
   const int n = 4;
   Mesh mesh = Mesh::MakeCartesian3D(n, n, n, Element::HEXAHEDRON, 1.0, 1.0, 1.0, true);
   jitter_vertices(mesh, n, 0.1, 1);
   g_modes = make_modes(3);
   FunctionCoefficient kfn(kappa_fn);
   const int orders[3] = {1, 2, 4};
   const int L = 3;
   Array<int> ess_bdr(mesh.bdr_attributes.Max());
   ess_bdr = 1;
   std::vector<H1_FECollection *> fecs;
   std::vector<FiniteElementSpace *> spaces;
   std::vector<BilinearForm *> forms;
   std::vector<Array<int>> ess(L);
   Array<Operator *> ops, prolongs;
   Array<Solver *> smoothers;
   Array<bool> own_ops, own_sm, own_pr;
   std::vector<double> lambdas;
   for (int l = 0; l < L; l++)
   {
      fecs.push_back(new H1_FECollection(orders[l], 3));
      spaces.push_back(new FiniteElementSpace(&mesh, fecs.back()));
      FiniteElementSpace &fes = *spaces.back();
      const std::string lv = "l" + std::to_string(l) + "_";
      // the default rule of DiffusionIntegrator::GetRule (fem/bilininteg.cpp:
      // 1346-1375): order 2p + 2, p + 2 points per direction
      const int q = orders[l] + 2;
      const IntegrationRule &ir = IntRules.Get(Geometry::CUBE, 2 * orders[l] + 2);
      MFEM_VERIFY(ir.GetNPoints() == q * q * q, "rule size");
      {
         const ElementRestriction *R = dynamic_cast<const ElementRestriction*>(
            fes.GetElementRestriction(ElementDofOrdering::LEXICOGRAPHIC));
         save(dir, (lv + "gather_map").c_str(), R->GatherMap());
         save(dir, (lv + "offsets").c_str(), R->Offsets());
         save(dir, (lv + "indices").c_str(), R->Indices());
         const DofToQuad &maps = fes.GetTypicalFE()->GetDofToQuad(ir, DofToQuad::TENSOR);
         save(dir, (lv + "B").c_str(), maps.B);
         save(dir, (lv + "G").c_str(), maps.G);
         const GeometricFactors *geom = mesh.GetGeometricFactors(ir, GeometricFactors::JACOBIANS);
         QuadratureSpace qs(mesh, ir);
         CoefficientVector cv(qs, CoefficientStorage::COMPRESSED);
         cv.Project(kfn);
         Vector qd(6 * q * q * q * mesh.GetNE());
         internal::PADiffusionSetup(3, 3, orders[l] + 1, q, 1, mesh.GetNE(), ir.GetWeights(), geom->J,
                                    cv, qd);
         save(dir, (lv + "qdata").c_str(), qd);
         if (l > 0)
         {
            // the transfer's tables: the coarse basis at this level's nodes
            // in lexicographic order (fem/transfer.cpp:2640-2656)
            const TensorBasisElement *htel =
               dynamic_cast<const TensorBasisElement*>(fes.GetTypicalFE());
            const Array<int> &hmap = htel->GetDofMap();
            const IntegrationRule &nodes = fes.GetTypicalFE()->GetNodes();
            IntegrationRule lex = nodes;
            for (int i = 0; i < nodes.GetNPoints(); ++i)
            {
               const int j = hmap[i] >= 0 ? hmap[i] : -1 - hmap[i];
               lex.IntPoint(i) = nodes.IntPoint(j);
            }
            const DofToQuad &tm = spaces[l - 1]->GetTypicalFE()->GetDofToQuad(lex, DofToQuad::TENSOR);
            save(dir, (lv + "Bi").c_str(), tm.B);
         }
      }
      BilinearForm *a = new BilinearForm(&fes);
      a->SetAssemblyLevel(AssemblyLevel::PARTIAL);
      a->AddDomainIntegrator(new DiffusionIntegrator(kfn, &ir));
      a->Assemble();
      forms.push_back(a);
      fes.GetEssentialTrueDofs(ess_bdr, ess[l]);
      OperatorPtr A;
      a->FormSystemMatrix(ess[l], A);
      A.SetOperatorOwner(false);
      ops.Append(A.Ptr()); own_ops.Append(true);
      save(dir, (lv + "ess").c_str(), ess[l]);
      if (l == 0)
      {
         CGSolver *cg = new CGSolver();
         cg->SetPrintLevel(-1);
         cg->SetMaxIter(200);
         cg->SetRelTol(sqrt(1e-4));
         cg->SetAbsTol(0.0);
         cg->SetOperator(*A.Ptr());
         smoothers.Append(cg);
      }
      else
      {
         Vector diag(fes.GetTrueVSize());
         a->AssembleDiagonal(diag);
         save(dir, (lv + "diag").c_str(), diag);
         // the smoother's own eigenvalue estimate, repeated to record it
         OperatorJacobiSmoother invd(diag, ess[l], 1.0);
         ProductOperator dA(&invd, A.Ptr(), false, false);
         PowerMethod pm;
         Vector ev(fes.GetTrueVSize());
         const double lam = pm.EstimateLargestEigenvalue(dA, ev, 10, 1e-8, 12345);
         lambdas.push_back(lam);
         smoothers.Append(new OperatorChebyshevSmoother(*A.Ptr(), diag, ess[l], 2));
         // the smoother applied with the recorded estimate to a fixed vector
         OperatorChebyshevSmoother S(*A.Ptr(), diag, ess[l], 2, lam);
         Vector x(fes.GetTrueVSize()), y(fes.GetTrueVSize());
         uint64_t sd = 20 + l;
         for (int i = 0; i < x.Size(); i++) { x(i) = 2.0 * u01(sd) - 1.0; }
         S.Mult(x, y);
         save(dir, (lv + "cheb_x").c_str(), x);
         save(dir, (lv + "cheb_y").c_str(), y);
      }
      own_sm.Append(true);
      if (l > 0)
      {
         TransferOperator *P = new TransferOperator(*spaces[l - 1], fes);
         prolongs.Append(P); own_pr.Append(true);
         Vector xc(spaces[l - 1]->GetTrueVSize()), yf(fes.GetTrueVSize());
         Vector xf(fes.GetTrueVSize()), yc(spaces[l - 1]->GetTrueVSize());
         uint64_t s1 = 30 + l, s2 = 40 + l;
         for (int i = 0; i < xc.Size(); i++) { xc(i) = 2.0 * u01(s1) - 1.0; }
         for (int i = 0; i < xf.Size(); i++) { xf(i) = 2.0 * u01(s2) - 1.0; }
         P->Mult(xc, yf);
         P->MultTranspose(xf, yc);
         save(dir, (lv + "P_x").c_str(), xc);
         save(dir, (lv + "P_y").c_str(), yf);
         save(dir, (lv + "Pt_x").c_str(), xf);
         save(dir, (lv + "Pt_y").c_str(), yc);
      }
   }
   save_dbls(dir, "lambda", lambdas);
   Multigrid mg(ops, smoothers, prolongs, own_ops, own_sm, own_pr);
   mg.SetCycleType(Multigrid::CycleType::VCYCLE, 1, 1);
   FiniteElementSpace &ffes = *spaces.back();
   ConstantCoefficient one(1.0);
   LinearForm b(&ffes);
   b.AddDomainIntegrator(new DomainLFIntegrator(one));
   b.Assemble();
   GridFunction xs(&ffes); xs = 0.0;
   OperatorPtr A; Vector X, Bv;
   forms.back()->FormLinearSystem(ess.back(), xs, b, A, X, Bv);
   save(dir, "B_rhs", Bv);
   {
      // one preconditioner application (V-cycle) to the right-hand side
      Vector Mb(Bv.Size());
      mg.Mult(Bv, Mb);
      save(dir, "mg_b", Mb);
   }
   CGSolver cg;
   cg.SetRelTol(1e-10); cg.SetAbsTol(0.0); cg.SetMaxIter(200); cg.SetPrintLevel(0);
   cg.SetOperator(*A); cg.SetPreconditioner(mg);
   X = 0.0;
   cg.Mult(Bv, X);
   save(dir, "X", X);
   std::vector<double> info = {(double)cg.GetNumIterations(), cg.GetFinalNorm(), (double)cg.GetConverged()};
   save_dbls(dir, "cg_info", info);
   std::vector<int> meta = {mesh.GetNE(), n, orders[0], orders[1], orders[2]};
   save_ints(dir, "meta", meta);
   printf("pmg4_p124: MG-PCG iterations %d final norm %.6e lambda %.6f %.6f\n", cg.GetNumIterations(),
          cg.GetFinalNorm(), lambdas[0], lambdas[1]);
   for (auto *f : forms) { delete f; }
   for (auto *f : spaces) { delete f; }
   for (auto *f : fecs) { delete f; }
}

int main(int argc, char **argv)
{
   if (argc < 2) { fprintf(stderr, "usage: %s outdir\n", argv[0]); return 1; }
   Device device("cpu");
   const std::string root = argv[1];
   mkdir(root.c_str(), 0755);
   const Case cases[] =
   {
      // name            n  p  q  jitter coeff    curved solve
      {"cart2_p2_one",    2, 2, 4, 0.0, C_ONE,    false, false},
      {"cart2_p1_const",  2, 1, 3, 0.0, C_CONST,  false, false},
      {"jit3_p3_fn",      3, 3, 5, 0.1, C_FN,     false, false},
      {"jit2_p4_vec",     2, 4, 6, 0.1, C_VEC,    false, false},
      {"jit2_p4_sym",     2, 4, 6, 0.1, C_SYM,    false, false},
      {"jit2_p2_nonsym",  2, 2, 4, 0.1, C_NONSYM, false, false},
      {"jit2_p6_fn",      2, 6, 8, 0.1, C_FN,     false, false},
      {"cart1_p8_one",    1, 8, 10, 0.0, C_ONE,   false, false},
      {"jit1_p7_fn",      1, 7, 9, 0.1, C_FN,     false, false},
      {"jit2_p5_fn",      2, 5, 7, 0.1, C_FN,     false, false},
      {"curv2_p5_fn",     2, 5, 7, 0.0, C_FN,     true,  false},
      {"curv2_p3_fn",     2, 3, 5, 0.0, C_FN,     true,  false},
      {"cfg1_solve",      8, 3, 4, 0.0, C_ONE,    false, true},
   };
   for (const Case &c : cases) { run_case(c, root); }
   run_pmg(root);
   return 0;
}
