"""Operator Mult on host buffers (gbpa_operator_mult_host): pinned buffers are
read and written by the kernels in place, pageable ones are staged; both must
give exactly the device Mult's result, for FP64, double-float and FP32
operators, with and without essential dofs."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def operator(precision, ess):
    from mfem_gb300 import fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, PAOperator
    from tests.gpu_util import dev
    dev()
    mesh = fem.CartesianMesh(5, jitter=0.1, seed=3)
    fes = FiniteElementSpace(mesh, 3)
    integ = DiffusionIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    e = fes.GetBoundaryTrueDofs() if ess else None
    return PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=e, precision=precision)


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("ess", [False, True])
@pytest.mark.parametrize("pin_x,pin_y", [(True, True), (False, False), (True, False), (False, True)])
def test_mult_host_equals_device_mult(precision, ess, pin_x, pin_y):
    A = operator(precision, ess)
    dt = torch.float32 if precision == 1 else torch.float64
    n = A.ndofs
    gen = torch.Generator().manual_seed(21)
    xh = (torch.rand(n, dtype=torch.float64, generator=gen) - 0.5).to(dt)
    hx = xh.pin_memory() if pin_x else xh.clone()
    hy = torch.full((n,), float("nan"), dtype=dt)
    if pin_y:
        hy = hy.pin_memory()
    A.MultHost(hx, hy)
    y = torch.empty(n, dtype=dt, device="cuda")
    A.Mult(xh.cuda(), y)
    torch.cuda.synchronize()
    assert torch.equal(hy, y.cpu())


def test_mult_host_repeated_and_rejects_device_tensors():
    A = operator(0, True)
    n = A.ndofs
    hx = torch.rand(n, dtype=torch.float64).pin_memory()
    hy = torch.empty(n, dtype=torch.float64).pin_memory()
    ref = torch.empty(n, dtype=torch.float64, device="cuda")
    A.Mult(hx.cuda(), ref)
    for _ in range(3):
        hy.zero_()
        A.MultHost(hx, hy)
        assert torch.equal(hy, ref.cpu())
    with pytest.raises(ValueError):
        A.MultHost(hx.cuda(), hy)
