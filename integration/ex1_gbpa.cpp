// The cfg1 Dirichlet Poisson problem written against MFEM's unchanged API, as
// an application would: unit cube, Mesh::MakeCartesian3D(8, 8, 8, HEXAHEDRON),
// H1 order 3 (Gauss-Lobatto), DiffusionIntegrator with coefficient 1 on the
// order-7 rule (2 (p + 1) - 1: 4 Gauss points per direction), f = 1,
// homogeneous Dirichlet on every boundary, AssemblyLevel::PARTIAL,
// FormLinearSystem, CGSolver + OperatorJacobiSmoother, rel. tol. 1e-12, at
// most 500 iterations (examples/ex1.cpp's structure).
//
// Linked to an MFEM whose PABilinearFormExtension carries the libgbpa hooks
// (integration/mfem_gbpa_patch.py); with MFEM_GBPA=1 every operator Mult of
// the solve runs in libgbpa on the GPU. Prints one JSON object: iterations,
// final norm, the number of forwarded Mult calls, whether libgbpa.so is mapped
// into this process (its /proc/self/maps line), and writes the solution X as
// raw doubles to argv[1].
#include "mfem.hpp"
#include "gbpa_shim.hpp"

#include <cstdio>
#include <fstream>
#include <string>

using namespace mfem;

int main(int argc, char **argv)
{
   if (argc < 2)
   {
      fprintf(stderr, "usage: %s <solution output file> [device]\n", argv[0]);
      return 2;
   }
   Device device(argc > 2 ? argv[2] : "cpu");
   const int n = 8, p = 3;
   Mesh mesh = Mesh::MakeCartesian3D(n, n, n, Element::HEXAHEDRON, 1.0, 1.0, 1.0, true);
   H1_FECollection fec(p, 3);
   FiniteElementSpace fes(&mesh, &fec);
   const IntegrationRule &ir = IntRules.Get(Geometry::CUBE, 2 * (p + 1) - 1);

   Array<int> ess_tdof_list, ess_bdr(mesh.bdr_attributes.Max());
   ess_bdr = 1;
   fes.GetEssentialTrueDofs(ess_bdr, ess_tdof_list);

   ConstantCoefficient one(1.0);
   LinearForm b(&fes);
   b.AddDomainIntegrator(new DomainLFIntegrator(one));
   b.Assemble();

   GridFunction x(&fes);
   x = 0.0;
   BilinearForm a(&fes);
   a.SetAssemblyLevel(AssemblyLevel::PARTIAL);
   a.AddDomainIntegrator(new DiffusionIntegrator(&ir));
   a.Assemble();

   OperatorPtr A;
   Vector X, B;
   a.FormLinearSystem(ess_tdof_list, x, b, A, X, B);
   OperatorJacobiSmoother M(a, ess_tdof_list);
   CGSolver cg;
   cg.SetRelTol(1e-12);
   cg.SetAbsTol(0.0);
   cg.SetMaxIter(500);
   cg.SetPrintLevel(0);
   cg.SetOperator(*A);
   cg.SetPreconditioner(M);
   cg.Mult(B, X);
   a.RecoverFEMSolution(X, b, x);

   {
      std::ofstream out(argv[1], std::ios::binary);
      const double *h = X.HostRead();
      out.write(reinterpret_cast<const char *>(h), sizeof(double) * X.Size());
   }
   std::string mapped;
   {
      std::ifstream maps("/proc/self/maps");
      std::string line;
      while (std::getline(maps, line))
      {
         if (line.find("libgbpa") != std::string::npos) { mapped = line.substr(line.find('/')); break; }
      }
   }
   printf("{\"iterations\": %d, \"final_norm\": %.17g, \"converged\": %d, \"ndofs\": %d, "
          "\"forwarded_mults\": %ld, \"libgbpa_mapped\": \"%s\"}\n",
          cg.GetNumIterations(), cg.GetFinalNorm(), cg.GetConverged() ? 1 : 0, X.Size(),
          gbpa_shim::ForwardedMults(), mapped.c_str());
   return 0;
}
