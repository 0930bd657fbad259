"""The 3D thread layout of the gather-fused diffusion apply (one thread per
quadrature point) against the 2D slab: the same multiply-adds in the same
order, so bit-identical results with the CSR scatter (to rounding with the
atomic one), for every order with a 3D kernel, the three arithmetics,
constrained or not."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu

DQ3_P = [1, 2, 3, 4, 5, 6, 7, 8]


def op(p, precision, ess, scatter=0, n=4):
    from mfem_gb300 import fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, PAOperator
    from tests.gpu_util import dev
    dev()
    mesh = fem.CartesianMesh(n, jitter=0.1, seed=9)
    fes = FiniteElementSpace(mesh, p)
    integ = DiffusionIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    e = fes.GetBoundaryTrueDofs() if ess else None
    A = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=e, precision=precision,
                   scatter=scatter)
    return fes, integ, A


def set_layout(d, precision, D, Q, layout, nbz, kind=0):
    return d.lib.gbpa_set_apply_layout(kind, precision, D, Q, layout, nbz)


def saved_layout(d, precision, D, Q, kind=0):
    """The installed (layout, nbz) of an order, to put back after a test."""
    n = ctypes.c_int(0)
    layout = d.lib.gbpa_get_apply_layout(kind, precision, D, Q, ctypes.byref(n))
    return layout, (n.value if layout == 1 else 0)


@pytest.mark.parametrize("p", DQ3_P)
@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("ess,scatter", [(False, 0), (True, 0), (True, 1)])
def test_3d_layout_matches_slab(p, precision, ess, scatter):
    from tests.gpu_util import dev
    d = dev()
    fes, integ, A = op(p, precision, ess, scatter)
    D, Q = integ.D, integ.Q
    dt = torch.float32 if precision == 1 else torch.float64
    gen = torch.Generator(device="cuda").manual_seed(61)
    x = (torch.rand(fes.ndofs, dtype=torch.float64, device="cuda", generator=gen) - 0.5).to(dt)
    y2, y3 = torch.empty_like(x), torch.full_like(x, float("nan"))
    nbz = max(1, min(4, 1024 // Q ** 3))
    before = saved_layout(d, precision, D, Q)
    assert set_layout(d, precision, D, Q, 0, 0) == 0
    try:
        A.Mult(x, y2)
        assert set_layout(d, precision, D, Q, 1, nbz) == 0
        n = ctypes.c_int(0)
        assert d.lib.gbpa_get_apply_layout(0, precision, D, Q, ctypes.byref(n)) == 1 and n.value == nbz
        A.Mult(x, y3)
        torch.cuda.synchronize()
    finally:
        set_layout(d, precision, D, Q, *before)
    if scatter == 0:
        # same multiply-adds in the same order (explicit FMAs): bit-identical
        assert torch.equal(y3, y2)
    else:
        tol = 1e-6 if precision == 1 else 1e-13
        assert float(torch.linalg.norm(y3 - y2) / torch.linalg.norm(y2)) < tol


def test_3d_layout_nbz_sweep_and_ragged_last_block():
    """Every feasible elements-per-block count gives the same result, including
    a last block with fewer elements than nbz (5^3 = 125 elements)."""
    from tests.gpu_util import dev
    d = dev()
    fes, integ, A = op(2, 0, True, n=5)
    D, Q = integ.D, integ.Q
    x = torch.rand(fes.ndofs, dtype=torch.float64, device="cuda")
    ref = torch.empty_like(x)
    before = saved_layout(d, 0, D, Q)
    try:
        set_layout(d, 0, D, Q, 0, 0)
        A.Mult(x, ref)
        for nbz in (1, 2, 3, 7, 64 // Q):
            assert set_layout(d, 0, D, Q, 1, nbz) == 0
            y = torch.full_like(x, float("nan"))
            A.Mult(x, y)
            torch.cuda.synchronize()
            assert float(torch.linalg.norm(y - ref) / torch.linalg.norm(ref)) < 1e-13, nbz
    finally:
        set_layout(d, 0, D, Q, *before)


@pytest.mark.parametrize("p", [1, 3, 5, 8])
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_3d_layout_mass_matches_slab(p, precision):
    from mfem_gb300 import fem
    from mfem_gb300.pa import FiniteElementSpace, MassIntegrator, PAOperator
    from tests.gpu_util import dev
    d = dev()
    mesh = fem.CartesianMesh(4, jitter=0.1, seed=9)
    fes = FiniteElementSpace(mesh, p)
    integ = MassIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    A = PAOperator(1, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=fes.GetBoundaryTrueDofs(),
                   precision=precision)
    D, Q = integ.D, integ.Q
    dt = torch.float32 if precision == 1 else torch.float64
    gen = torch.Generator(device="cuda").manual_seed(62)
    x = (torch.rand(fes.ndofs, dtype=torch.float64, device="cuda", generator=gen) - 0.5).to(dt)
    y2, y3 = torch.empty_like(x), torch.full_like(x, float("nan"))
    nbz = max(1, min(4, 1024 // Q ** 3, 64 // Q))
    before = saved_layout(d, precision, D, Q, kind=1)
    try:
        assert set_layout(d, precision, D, Q, 0, 0, kind=1) == 0
        A.Mult(x, y2)
        assert set_layout(d, precision, D, Q, 1, nbz, kind=1) == 0
        A.Mult(x, y3)
        torch.cuda.synchronize()
    finally:
        set_layout(d, precision, D, Q, *before, kind=1)
    assert torch.equal(y3, y2)


def test_layout_arguments_validated():
    from tests.gpu_util import dev
    d = dev()
    assert d.lib.gbpa_set_apply_layout(2, 0, 4, 5, 1, 1) == -1      # unknown kind
    assert d.lib.gbpa_set_apply_layout(0, 0, 4, 5, 3, 1) == -1      # unknown layout
    assert d.lib.gbpa_set_apply_layout(0, 0, 4, 5, 2, 1) == -2      # tensor-core layout: FP32 only
    assert d.lib.gbpa_set_apply_layout(0, 0, 4, 5, 1, 0) == -1      # nbz < 1
    assert d.lib.gbpa_set_apply_layout(0, 0, 9, 10, 1, 2) == -1     # 2000 threads
    assert d.lib.gbpa_set_apply_layout(0, 0, 2, 3, 1, 30) == -1     # blockDim.z = 90 > 64
    assert d.lib.gbpa_get_apply_layout(0, 0, 4, 5, None) == 0
