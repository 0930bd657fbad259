"""The atomic scatter (GBPA_SCATTER_ATOMIC: the element kernel adds its results
into the L-vector through the gather map, no E-vector) against the
deterministic CSR scatter: same operator to rounding (the summation order
differs), same PCG and mixed-precision solutions."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def operators(kind, precision, ess, n=5, p=3):
    from mfem_gb300 import _lib, fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, MassIntegrator, PAOperator
    from tests.gpu_util import dev
    dev()
    mesh = fem.CartesianMesh(n, jitter=0.1, seed=7)
    fes = FiniteElementSpace(mesh, p)
    integ = DiffusionIntegrator("kappa") if kind == 0 else MassIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    e = fes.GetBoundaryTrueDofs() if ess else None
    qd = integ.qdata
    mk = lambda sc: PAOperator(kind, fes, integ.D, integ.Q, integ.B, getattr(integ, "G", integ.B), qd,
                               ess=e, precision=precision, scatter=sc)
    return fes, e, mk(_lib.GBPA_SCATTER_CSR), mk(_lib.GBPA_SCATTER_ATOMIC)


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("ess", [False, True])
def test_atomic_mult_matches_csr(kind, precision, ess):
    fes, e, Acsr, Aat = operators(kind, precision, ess)
    dt = torch.float32 if precision == 1 else torch.float64
    gen = torch.Generator(device="cuda").manual_seed(51)
    x = (torch.rand(fes.ndofs, dtype=torch.float64, device="cuda", generator=gen) - 0.5).to(dt)
    y0, y1 = torch.empty_like(x), torch.full_like(x, float("nan"))
    Acsr.Mult(x, y0)
    Aat.Mult(x, y1)
    tol = 1e-6 if precision == 1 else 1e-14
    assert float(torch.linalg.norm(y1 - y0) / torch.linalg.norm(y0)) < tol
    if ess:
        idx = torch.from_numpy(e).long().cuda()
        assert torch.equal(y1[idx], x[idx])


def test_atomic_mult_rejects_in_place():
    from tests.gpu_util import dev
    fes, _, _, Aat = operators(0, 0, True)
    x = torch.rand(fes.ndofs, dtype=torch.float64, device="cuda")
    assert dev().lib.gbpa_operator_mult(Aat.handle, ctypes.c_void_p(x.data_ptr()),
                                        ctypes.c_void_p(x.data_ptr())) == -1


def test_atomic_pcg_and_mixed_reliable_match_csr():
    from mfem_gb300 import _lib
    from mfem_gb300.pa import OperatorJacobiSmoother, PAOperator
    from tests.gpu_util import dev
    d = dev()
    fes, e, A64, A64a = operators(0, 0, True, n=8, p=4)
    _, _, A32, A32a = operators(0, 1, True, n=8, p=4)
    M = OperatorJacobiSmoother(A64, e)
    gen = torch.Generator(device="cuda").manual_seed(52)
    b = torch.rand(fes.ndofs, dtype=torch.float64, device="cuda", generator=gen)
    b[torch.from_numpy(e).long().cuda()] = 0.0
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    x0, x1 = torch.zeros_like(b), torch.zeros_like(b)
    i0, i1 = _lib.SolveInfo(), _lib.SolveInfo()
    assert d.lib.gbpa_pcg_solve(A64.handle, P(M.dinv), P(b), P(x0), 1e-12, 0.0, 5000, 0, ctypes.byref(i0)) == 0
    assert d.lib.gbpa_pcg_solve(A64a.handle, P(M.dinv), P(b), P(x1), 1e-12, 0.0, 5000, 0, ctypes.byref(i1)) == 0
    assert abs(i0.iterations - i1.iterations) <= 3
    assert float(torch.linalg.norm(x1 - x0) / torch.linalg.norm(x0)) < 1e-10
    xr = torch.zeros_like(b)
    ir = _lib.SolveInfo()
    assert d.lib.gbpa_pcg_solve_mixed_reliable(A64a.handle, A32a.handle, P(M.dinv.float()), P(b), P(xr),
                                               1e-10, 0.1, 5000, ctypes.byref(ir)) == 0
    assert ir.converged == 1 and ir.true_rel_residual <= 1e-10
    assert float(torch.linalg.norm(xr - x0) / torch.linalg.norm(x0)) < 1e-8
