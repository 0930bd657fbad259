"""PCG on the device against the reference's own solve of the Dirichlet
Poisson problem (unit cube, 8^3 hexes, p = 3, Q = 4, f = 1, PCG + Jacobi,
rel tol 1e-12): solution within 1e-10 relative L2, same iteration count
(+-1). The mixed-precision form must reach the FP64 solution within 1e-9."""
import numpy as np
import pytest
import torch

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def cfg1_operator():
    from mfem_gb300.pa import ElementRestriction, PAOperator
    from tests.gpu_util import T, p, call, zeros, dev
    dev()
    g = load_golden("cfg1_solve")
    ne, ndofs, D, Q = (int(v) for v in g["meta"][:4])
    qd = zeros(Q ** 3 * 6 * ne)
    C = T(g["coeff"])
    call("gbpa_diffusion_setup3d_nodes", ne, 2, Q, 1, p(T(g["W"])), p(T(g["Bg"])), p(T(g["Gg"])),
         p(T(g["nodesE"])), p(C), C.numel(), p(qd))
    R = ElementRestriction.from_maps(ne, D ** 3, ndofs, g["gather_map"], g["offsets"], g["indices"])
    A = PAOperator(0, R, D, Q, T(g["B"]), T(g["G"]), qd, ess=g["ess_tdofs"])
    A32 = PAOperator(0, R, D, Q, T(g["B"]), T(g["G"]), qd, ess=g["ess_tdofs"], precision=1)
    return g, ndofs, A, A32


def jacobi(g, A, ndofs):
    from tests.gpu_util import T, p, call, zeros
    diag = zeros(ndofs)
    A.AssembleDiagonal(diag)
    dinv = zeros(ndofs)
    ess = T(g["ess_tdofs"])
    call("gbpa_jacobi_setup", ndofs, p(diag), p(ess), ess.numel(), 1.0, p(dinv))
    return diag, dinv


def test_constrained_operator_and_jacobi():
    from tests.gpu_util import T, H, zeros, relerr
    g, ndofs, A, _ = cfg1_operator()
    y = zeros(ndofs)
    A.Mult(T(g["x"]), y)
    assert relerr(H(y), g["Ax_constrained"]) < 1e-12
    diag, dinv = jacobi(g, A, ndofs)
    assert relerr(H(dinv) * g["x"], g["Mx_jacobi"]) < 1e-12


def test_pcg_matches_reference_solve():
    import ctypes
    from mfem_gb300 import _lib
    from tests.gpu_util import T, H, p, zeros, relerr, dev
    g, ndofs, A, _ = cfg1_operator()
    _, dinv = jacobi(g, A, ndofs)
    X = zeros(ndofs)
    info = _lib.SolveInfo()
    st = dev().lib.gbpa_pcg_solve(A.handle, p(dinv), p(T(g["B_rhs"])), p(X), 1e-12, 0.0, 500, 0,
                                  ctypes.byref(info))
    assert st == 0
    ref_it, ref_norm, ref_conv = g["cg_info"]
    assert info.converged == 1
    assert abs(info.iterations - int(ref_it)) <= 1
    # the last preconditioned residual is rounding-dominated at 1e-12: check
    # the stopping rule and the order of magnitude, not its digits
    assert info.final_norm <= 1e-12 * info.initial_norm
    assert 0.5 * ref_norm <= info.final_norm <= 2.0 * ref_norm
    assert relerr(H(X), g["X"]) < 1e-10
    assert info.true_rel_residual < 1e-10
    # iterative mode (linalg/solvers.cpp:875-879) from the converged solution:
    # r0 = b - A x is already at the converged level, and an absolute
    # tolerance just above it stops the solve at once, on the same solution
    first_initial = info.initial_norm
    st = dev().lib.gbpa_pcg_solve(A.handle, p(dinv), p(T(g["B_rhs"])), p(X), 0.0, 1e-8 * first_initial,
                                  500, 1, ctypes.byref(info))
    assert st == 0 and info.converged == 1 and info.iterations == 0
    assert info.initial_norm <= 1e-8 * first_initial
    assert relerr(H(X), g["X"]) < 1e-10


def test_mixed_precision_matches_reference_solve():
    import ctypes
    from mfem_gb300 import _lib
    from tests.gpu_util import T, H, p, zeros, relerr, dev
    g, ndofs, A, A32 = cfg1_operator()
    _, dinv = jacobi(g, A, ndofs)
    X = zeros(ndofs)
    info = _lib.SolveInfo()
    st = dev().lib.gbpa_pcg_solve_mixed(A.handle, A32.handle, p(dinv.float()), p(T(g["B_rhs"])), p(X),
                                        1e-10, 1e-5, 20, 500, ctypes.byref(info))
    assert st == 0, info.as_dict()
    assert info.converged == 1 and info.true_rel_residual <= 1e-10
    assert relerr(H(X), g["X"]) < 1e-9
    assert info.outer_iterations >= 2


@pytest.mark.parametrize("delta", [0.1, 0.01])
def test_mixed_reliable_matches_reference_solve(delta):
    """One FP32 PCG with FP64 residual replacement: the reference's solution
    within 1e-9, true residual within the tolerance, FP32 iterations close to
    the reference's FP64 count (no Krylov restarts)."""
    import ctypes
    from mfem_gb300 import _lib
    from tests.gpu_util import T, H, p, zeros, relerr, dev
    g, ndofs, A, A32 = cfg1_operator()
    _, dinv = jacobi(g, A, ndofs)
    X = zeros(ndofs)
    info = _lib.SolveInfo()
    st = dev().lib.gbpa_pcg_solve_mixed_reliable(A.handle, A32.handle, p(dinv.float()), p(T(g["B_rhs"])),
                                                 p(X), 1e-10, delta, 1000, ctypes.byref(info))
    assert st == 0, info.as_dict()
    assert info.converged == 1 and info.true_rel_residual <= 1e-10
    assert relerr(H(X), g["X"]) < 1e-9
    assert info.outer_iterations >= 2
    assert info.iterations <= 1.3 * int(g["cg_info"][0]) + 10


def test_mixed_reliable_on_jittered_lognormal_problem():
    """A harder case (jittered p=4 mesh, lognormal kappa): the reliable mixed
    solution matches FP64 PCG to 1e-8 and needs no more FP32 iterations than
    the restarted defect correction."""
    import ctypes
    from mfem_gb300 import _lib, fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, OperatorJacobiSmoother, PAOperator
    from tests.gpu_util import dev
    d = dev()
    mesh = fem.CartesianMesh(10, jitter=0.1, seed=1)
    fes = FiniteElementSpace(mesh, 4)
    integ = DiffusionIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    e = fes.GetBoundaryTrueDofs()
    A = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=e)
    A32 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=e, precision=1)
    M = OperatorJacobiSmoother(A, e)
    n = fes.ndofs
    gen = torch.Generator(device="cuda").manual_seed(41)
    b = torch.rand(n, dtype=torch.float64, device="cuda", generator=gen)
    b[torch.from_numpy(e).long().cuda()] = 0.0
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    x64 = torch.zeros_like(b)
    i64 = _lib.SolveInfo()
    assert d.lib.gbpa_pcg_solve(A.handle, P(M.dinv), P(b), P(x64), 1e-12, 0.0, 20000, 0, ctypes.byref(i64)) == 0
    dinv32 = M.dinv.float()
    xr = torch.zeros_like(b)
    ir = _lib.SolveInfo()
    assert d.lib.gbpa_pcg_solve_mixed_reliable(A.handle, A32.handle, P(dinv32), P(b), P(xr), 1e-10, 0.1,
                                               20000, ctypes.byref(ir)) == 0
    xm = torch.zeros_like(b)
    im = _lib.SolveInfo()
    assert d.lib.gbpa_pcg_solve_mixed(A.handle, A32.handle, P(dinv32), P(b), P(xm), 1e-10, 1e-5, 30, 20000,
                                      ctypes.byref(im)) == 0
    assert ir.converged == 1 and ir.true_rel_residual <= 1e-10
    assert float(torch.linalg.norm(xr - x64) / torch.linalg.norm(x64)) < 1e-8
    assert ir.iterations <= im.inner_iterations


def test_mixed_reliable_rejects_bad_arguments():
    import ctypes
    from mfem_gb300 import _lib
    from tests.gpu_util import T, p, zeros, dev
    g, ndofs, A, A32 = cfg1_operator()
    _, dinv = jacobi(g, A, ndofs)
    X = zeros(ndofs)
    info = _lib.SolveInfo()
    lib = dev().lib
    b = T(g["B_rhs"])
    for delta in (0.0, 1.0, -0.5):
        assert lib.gbpa_pcg_solve_mixed_reliable(A.handle, A32.handle, p(dinv.float()), p(b), p(X), 1e-10,
                                                 delta, 100, ctypes.byref(info)) == -1
    # operators swapped (the FP32 one must be second)
    assert lib.gbpa_pcg_solve_mixed_reliable(A32.handle, A.handle, p(dinv.float()), p(b), p(X), 1e-10,
                                             0.1, 100, ctypes.byref(info)) == -1
    # iteration cap: not converged, reported as such
    st = lib.gbpa_pcg_solve_mixed_reliable(A.handle, A32.handle, p(dinv.float()), p(b), p(X), 1e-10,
                                           0.1, 5, ctypes.byref(info))
    assert st == -6 and info.converged == 0


def test_max_iterations_not_converged():
    import ctypes
    from mfem_gb300 import _lib
    from tests.gpu_util import T, p, zeros, dev
    g, ndofs, A, _ = cfg1_operator()
    _, dinv = jacobi(g, A, ndofs)
    X = zeros(ndofs)
    info = _lib.SolveInfo()
    st = dev().lib.gbpa_pcg_solve(A.handle, p(dinv), p(T(g["B_rhs"])), p(X), 1e-12, 0.0, 5, 0,
                                  ctypes.byref(info))
    assert st == 0 and info.converged == 0 and info.iterations == 5


def test_double_float_pcg_matches_reference_solve():
    import ctypes
    from mfem_gb300 import _lib
    from mfem_gb300.pa import ElementRestriction, PAOperator
    from tests.gpu_util import T, H, p, zeros, relerr, dev
    g, ndofs, A, _ = cfg1_operator()
    ne, _, D, Q = (int(v) for v in g["meta"][:4])
    R = ElementRestriction.from_maps(ne, D ** 3, ndofs, g["gather_map"], g["offsets"], g["indices"])
    A2 = PAOperator(0, R, D, Q, A.B, A.G, A.qdata, ess=g["ess_tdofs"], precision=2)
    _, dinv = jacobi(g, A, ndofs)
    X = zeros(ndofs)
    info = _lib.SolveInfo()
    st = dev().lib.gbpa_pcg_solve(A2.handle, p(dinv), p(T(g["B_rhs"])), p(X), 1e-12, 0.0, 500, 0,
                                  ctypes.byref(info))
    assert st == 0 and info.converged == 1
    assert abs(info.iterations - int(g["cg_info"][0])) <= 1
    assert relerr(H(X), g["X"]) < 1e-10
