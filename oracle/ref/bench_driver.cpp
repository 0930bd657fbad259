// CPU baseline driver: times the UNMODIFIED reference MFEM's own partial-
// assembly diffusion operator, BilinearForm::Mult with
// AssemblyLevel::PARTIAL (fem/bilinearform_ext.cpp:487-564), on the host cores
// through Device("omp") (the OpenMP forall backend, general/forall.hpp) or
// Device("cpu") (one thread). The library is the serial CPU build that
// oracle/ref/Makefile makes from the reference sources; this file only calls
// the reference's public API.
//
// Workload: the unit cube meshed by Mesh::MakeCartesian3D(n, n, n, HEXAHEDRON)
// with interior vertices moved by U(-0.1h, 0.1h) per coordinate (splitmix64,
// seed 1, three draws per vertex in vertex order -- the recipe of the GPU
// package's CartesianMesh, so both build the same geometry), H1 order p
// (Gauss-Lobatto), DiffusionIntegrator with coefficient 1 on its default rule
// (order 2p + dim - 1: p + 2 Gauss points per direction), x ~ U[-1, 1]
// (splitmix64, seed 2).
//
// Usage: bench_driver n p steps warmup [omp|cpu]
// Prints one JSON object: ndofs, ne, q1d, set-up seconds, per-apply seconds
// (median and total over `steps` timed applies), the OpenMP thread count and
// the checksum sum(y) of the last apply.
#include "mfem.hpp"
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace mfem;

static uint64_t splitmix64(uint64_t &s)
{
   uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
   z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
   z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
   return z ^ (z >> 31);
}
static double u01(uint64_t &s) { return (splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

static double now()
{
   return std::chrono::duration<double>(
             std::chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char **argv)
{
   if (argc < 5)
   {
      fprintf(stderr, "usage: %s n p steps warmup [omp|cpu]\n", argv[0]);
      return 2;
   }
   const int n = atoi(argv[1]), p = atoi(argv[2]);
   const int steps = atoi(argv[3]), warmup = atoi(argv[4]);
   const char *backend = argc > 5 ? argv[5] : "omp";
   if (n < 1 || p < 1 || steps < 1 || warmup < 0) { return 2; }
   Device device(backend);

   const double t0 = now();
   Mesh mesh = Mesh::MakeCartesian3D(n, n, n, Element::HEXAHEDRON, 1.0, 1.0, 1.0, true);
   {
      const double h = 1.0 / n, amp = 0.1;
      uint64_t s = 1;
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
   H1_FECollection fec(p, 3);
   FiniteElementSpace fes(&mesh, &fec);
   const int ndofs = fes.GetNDofs();
   BilinearForm a(&fes);
   a.SetAssemblyLevel(AssemblyLevel::PARTIAL);
   a.AddDomainIntegrator(new DiffusionIntegrator);
   a.Assemble();
   Vector x(ndofs), y(ndofs);
   {
      uint64_t s = 2;
      double *hx = x.HostWrite();
      for (int i = 0; i < ndofs; i++) { hx[i] = 2.0 * u01(s) - 1.0; }
   }
   x.UseDevice(true);
   y.UseDevice(true);
   const double setup = now() - t0;

   for (int i = 0; i < warmup; i++) { a.Mult(x, y); }
   std::vector<double> ts(steps);
   const double tt = now();
   for (int i = 0; i < steps; i++)
   {
      const double a0 = now();
      a.Mult(x, y);
      ts[i] = now() - a0;
   }
   const double total = now() - tt;
   std::vector<double> sorted = ts;
   std::sort(sorted.begin(), sorted.end());
   double sum = 0.0;
   const double *hy = y.HostRead();
   for (int i = 0; i < ndofs; i++) { sum += hy[i]; }
   int threads = 1;
#ifdef _OPENMP
   if (!strcmp(backend, "omp")) { threads = omp_get_max_threads(); }
#endif
   const IntegrationRule &ir = IntRules.Get(Geometry::CUBE, 2 * p + 3 - 1);
   int q1d = 1;
   while (q1d * q1d * q1d < ir.GetNPoints()) { q1d++; }
   printf("{\"ndofs\": %d, \"ne\": %d, \"p\": %d, \"q1d\": %d, \"backend\": \"%s\", "
          "\"threads\": %d, \"setup_s\": %.6f, \"steps\": %d, \"warmup\": %d, "
          "\"total_s\": %.6f, \"median_s\": %.6f, \"min_s\": %.6f, \"sum_y\": %.17g}\n",
          ndofs, mesh.GetNE(), p, q1d, backend, threads, setup, steps, warmup, total,
          sorted[steps / 2], sorted[0], sum);
   return 0;
}
