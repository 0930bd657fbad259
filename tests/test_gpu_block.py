"""Several right-hand sides (combined form): the block apply must equal R
single applies, the block PCG must reproduce R single PCG solves, and the
block mixed-precision solve must reach the FP64 solutions -- including on a
curved order-3 geometry."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def problem(n, p, curved=False, coeff="kappa", ess=True):
    from mfem_gb300 import fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, OperatorJacobiSmoother, PAOperator
    from tests.gpu_util import dev
    dev()
    mesh = fem.CartesianMesh(n, jitter=0.0 if curved else 0.1, seed=1, curved=curved)
    fes = FiniteElementSpace(mesh, p)
    integ = DiffusionIntegrator(coeff)
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    e = fes.GetBoundaryTrueDofs() if ess else None
    A = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=e)
    A32 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=e, precision=1)
    M = OperatorJacobiSmoother(A, e if e is not None else [])
    return fes, integ, A, A32, M, e


def P(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("R", [1, 2, 8])
@pytest.mark.parametrize("prec", [0, 1])
def test_block_mult_equals_single(R, prec):
    from tests.gpu_util import dev
    d = dev()
    fes, integ, A, A32, M, _ = problem(5, 3)
    op = A if prec == 0 else A32
    dt = torch.float64 if prec == 0 else torch.float32
    n = fes.ndofs
    gen = torch.Generator(device="cuda").manual_seed(11)
    X = (torch.rand(n, R, dtype=torch.float64, device="cuda", generator=gen) - 0.5).to(dt).contiguous()
    Y = torch.empty_like(X)
    assert d.lib.gbpa_operator_mult_block(op.handle, R, P(X), P(Y)) == 0
    # the single applies in the block kernel's family: at this order (no
    # tensor-core block kernel) the CUDA-core one, whatever the FP32 default
    D, Q = integ.D, integ.Q
    nb = ctypes.c_int(0)
    prev = d.lib.gbpa_get_apply_layout(0, prec, D, Q, ctypes.byref(nb))
    if prec == 1 and d.lib.gbpa_get_block_apply_layout(D, Q, R) == 0:
        assert d.lib.gbpa_set_apply_layout(0, 1, D, Q, 0, 0) == 0
    try:
        for r in range(R):
            y = torch.empty(n, dtype=dt, device="cuda")
            op.Mult(X[:, r].contiguous(), y)
            if prec == 0:
                assert torch.equal(Y[:, r], y)
            else:
                assert float(torch.linalg.norm(Y[:, r] - y) / torch.linalg.norm(y)) < 1e-6
    finally:
        d.lib.gbpa_set_apply_layout(0, prec, D, Q, prev, nb.value)


@pytest.mark.parametrize("R", [1, 2, 4, 8])
def test_block_pcg_matches_single_solves(R):
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    fes, integ, A, A32, M, e = problem(4, 4)
    n = fes.ndofs
    gen = torch.Generator(device="cuda").manual_seed(12)
    B = torch.rand(n, R, dtype=torch.float64, device="cuda", generator=gen)
    B[torch.from_numpy(e).long().cuda()] = 0.0
    B = B.contiguous()
    X = torch.zeros_like(B)
    info = (_lib.SolveInfo * R)()
    assert d.lib.gbpa_pcg_solve_block(A.handle, R, P(M.dinv), P(B), P(X), 1e-10, 0.0, 2000, info) == 0
    for r in range(R):
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        si = _lib.SolveInfo()
        b = B[:, r].contiguous()
        assert d.lib.gbpa_pcg_solve(A.handle, P(M.dinv), P(b), P(x), 1e-10, 0.0, 2000, 0, ctypes.byref(si)) == 0
        assert info[r].converged == 1 and abs(info[r].iterations - si.iterations) <= 1
        assert float(torch.linalg.norm(X[:, r] - x) / torch.linalg.norm(x)) < 1e-10


@pytest.mark.parametrize("curved", [False, True])
def test_block_mixed_reaches_fp64_solution(curved):
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    fes, integ, A, A32, M, e = problem(4, 5 if curved else 3, curved=curved)
    n, R = fes.ndofs, 8
    gen = torch.Generator(device="cuda").manual_seed(13)
    B = (torch.rand(n, R, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1)
    B[torch.from_numpy(e).long().cuda()] = 0.0
    B = B.contiguous()
    X = torch.zeros_like(B)
    info = (_lib.SolveInfo * R)()
    st = d.lib.gbpa_pcg_solve_block_mixed(A.handle, A32.handle, R, P(M.dinv.float()), P(B), P(X),
                                          1e-10, 1e-5, 20, 2000, info)
    assert st == 0
    X64 = torch.zeros_like(B)
    info64 = (_lib.SolveInfo * R)()
    assert d.lib.gbpa_pcg_solve_block(A.handle, R, P(M.dinv), P(B), P(X64), 1e-12, 0.0, 5000, info64) == 0
    for r in range(R):
        assert info[r].converged == 1 and info[r].true_rel_residual <= 1e-10
        assert float(torch.linalg.norm(X[:, r] - X64[:, r]) / torch.linalg.norm(X64[:, r])) < 1e-8


def test_curved_geometry_operator_against_oracle():
    """Order-3 curved geometry: the device Jacobians from order-3 nodes feed
    the same qdata as the oracle's restatement of the reference's
    geometric-factor and setup kernels."""
    from mfem_gb300 import fem
    from tests import oracle_lib
    fes, integ, A, _, _, _ = problem(3, 2, curved=True, coeff=None, ess=False)
    o = oracle_lib.load()
    mesh = fes.mesh
    gt = fem.Tables(3, integ.Q)
    J = o.geom_jacobians3d(fes.ne, 4, integ.Q, gt.B, gt.G, mesh.nodes_evector(3))
    qd = o.diffusion_setup3d(fes.ne, integ.Q, 1, integ.W.cpu().numpy(), J, np.array([1.0]))
    assert np.linalg.norm(integ.qdata.cpu().numpy() - qd) / np.linalg.norm(qd) < 1e-13


@pytest.mark.parametrize("curved", [False, True])
def test_block_mixed_reliable_reaches_fp64_solution(curved):
    """Block reliable-update mixed solve: every right-hand side converges on
    its true FP64 residual and matches the FP64 block solution; a zero
    right-hand side returns x = 0."""
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    fes, integ, A, A32, M, e = problem(4, 5 if curved else 3, curved=curved)
    n, R = fes.ndofs, 8
    gen = torch.Generator(device="cuda").manual_seed(14)
    B = (torch.rand(n, R, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1)
    B[torch.from_numpy(e).long().cuda()] = 0.0
    B[:, 3] = 0.0
    B = B.contiguous()
    X = torch.full_like(B, 7.0)
    info = (_lib.SolveInfo * R)()
    st = d.lib.gbpa_pcg_solve_block_mixed_reliable(A.handle, A32.handle, R, P(M.dinv.float()), P(B), P(X),
                                                   1e-10, 0.1, 5000, info)
    assert st == 0
    X64 = torch.zeros_like(B)
    info64 = (_lib.SolveInfo * R)()
    assert d.lib.gbpa_pcg_solve_block(A.handle, R, P(M.dinv), P(B), P(X64), 1e-12, 0.0, 5000, info64) == 0
    for r in range(R):
        assert info[r].converged == 1 and info[r].true_rel_residual <= 1e-10
        if r == 3:
            assert float(torch.abs(X[:, r]).max()) == 0.0
            continue
        assert float(torch.linalg.norm(X[:, r] - X64[:, r]) / torch.linalg.norm(X64[:, r])) < 1e-8
        assert info[r].outer_iterations >= 1


def test_block_mixed_reliable_matches_single_reliable():
    """R = 2: each column of the block solve equals the single-vector
    reliable solve of that column to 1e-9 (same algorithm, lockstep)."""
    import ctypes
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    fes, integ, A, A32, M, e = problem(4, 4)
    n, R = fes.ndofs, 2
    gen = torch.Generator(device="cuda").manual_seed(15)
    B = torch.rand(n, R, dtype=torch.float64, device="cuda", generator=gen)
    B[torch.from_numpy(e).long().cuda()] = 0.0
    B = B.contiguous()
    X = torch.zeros_like(B)
    info = (_lib.SolveInfo * R)()
    d32 = M.dinv.float()
    assert d.lib.gbpa_pcg_solve_block_mixed_reliable(A.handle, A32.handle, R, P(d32), P(B), P(X), 1e-10, 0.1,
                                                     5000, info) == 0
    for r in range(R):
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        si = _lib.SolveInfo()
        b = B[:, r].contiguous()
        assert d.lib.gbpa_pcg_solve_mixed_reliable(A.handle, A32.handle, P(d32), P(b), P(x), 1e-10, 0.1, 5000,
                                                   ctypes.byref(si)) == 0
        assert float(torch.linalg.norm(X[:, r] - x) / torch.linalg.norm(x)) < 1e-9
