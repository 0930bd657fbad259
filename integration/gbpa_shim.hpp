// Forwarding layer between MFEM's partial-assembly bilinear form and libgbpa.
//
// PABilinearFormExtension (fem/bilinearform_ext.cpp) calls these three hooks
// (mfem_gbpa_patch.py adds the calls; nothing else in MFEM changes):
//   Assemble  at the end of PABilinearFormExtension::Assemble: when the form
//             is one DiffusionIntegrator without element markers on a 3D
//             tensor-product H1 space, a libgbpa operator is created from
//             MFEM's own arrays -- the lexicographic ElementRestriction's
//             gather map and CSR transpose, the integrator's B, G and PA data
//             -- unchanged;
//   Mult      at the start of PABilinearFormExtension::MultInternal: y = A x
//             through libgbpa (restriction, sum-factorised apply and
//             transpose on the GPU); returns false when the form is not
//             forwarded, and MFEM's own path runs;
//   Release   in PABilinearFormExtension::Update: the space changed, the
//             operator is dropped.
// Forwarding is on when the environment variable MFEM_GBPA is "1"; the
// application's code (BilinearForm, SetAssemblyLevel(AssemblyLevel::PARTIAL),
// FormLinearSystem, CGSolver, OperatorJacobiSmoother) is unchanged.
#ifndef MFEM_GBPA_SHIM_HPP
#define MFEM_GBPA_SHIM_HPP

namespace mfem
{
class BilinearForm;
class Operator;
class Vector;

namespace gbpa_shim
{
bool Enabled();
void Assemble(const void *ext, BilinearForm &a, const Operator *elem_restrict);
bool Mult(const void *ext, BilinearForm &a, const Vector &x, Vector &y);
void Release(const void *ext);
// forwarded Mult calls so far in this process
long ForwardedMults();
} // namespace gbpa_shim
} // namespace mfem

#endif
