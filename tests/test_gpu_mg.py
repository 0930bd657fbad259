"""p-multigrid on the GPU (gbpa_ptransfer_*, gbpa_chebyshev_*,
gbpa_multigrid_*, gbpa_pcg_solve_mg) against the reference's own outputs on
the pmg4_p124 fixture (orders 1, 2, 4 on a jittered 4^3 mesh, lognormal
kappa) and against the CPU oracle; then the whole solve on larger meshes
against Jacobi-PCG on the same system."""
import ctypes

import numpy as np
import pytest
import torch

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu

ORDERS = (1, 2, 4)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


class GoldenHierarchy:
    """Operators, smoothers and transfers built from the fixture's own maps,
    tables and qdata through the C ABI."""

    def __init__(self, g, precision=0, lambdas=None):
        from mfem_gb300 import _lib
        from mfem_gb300.pa import ElementRestriction, PAOperator
        from tests.gpu_util import T, dev
        d = dev()
        self.d, self.g = d, g
        ne = int(g["meta"][0])
        self.R, self.ops, self.sm, self.P, self.diag = [], [], [None], [], [None]
        for l, p in enumerate(ORDERS):
            k = f"l{l}_"
            ndofs = g[k + "offsets"].size - 1
            R = ElementRestriction.from_maps(ne, (p + 1) ** 3, ndofs, g[k + "gather_map"], g[k + "offsets"],
                                             g[k + "indices"])
            A = PAOperator(0, R, p + 1, p + 2, T(g[k + "B"]), T(g[k + "G"]), T(g[k + "qdata"]), ess=g[k + "ess"],
                           precision=precision)
            self.R.append(R)
            self.ops.append(A)
            if l > 0:
                diag = T(g[k + "diag"])
                self.diag.append(diag)
                lam = float((g["lambda"] if lambdas is None else lambdas)[l - 1])
                h = ctypes.c_void_p()
                assert d.lib.gbpa_chebyshev_create(A.handle, ctypes.c_void_p(diag.data_ptr()), 2, lam, 10, 1e-8,
                                                   12345, ctypes.byref(h)) == 0
                self.sm.append(h)
                Rc = self.R[l - 1]
                Bi = np.ascontiguousarray(g[k + "Bi"])
                hp = ctypes.c_void_p()
                assert d.lib.gbpa_ptransfer_create(
                    d.ctx, ne, ORDERS[l - 1] + 1, Rc.ndofs, ctypes.c_void_p(Rc.gather_map.data_ptr()),
                    ctypes.c_void_p(Rc.offsets.data_ptr()), ctypes.c_void_p(Rc.indices.data_ptr()), p + 1,
                    ndofs, ctypes.c_void_p(R.gather_map.data_ptr()), ctypes.c_void_p(R.offsets.data_ptr()),
                    ctypes.c_void_p(R.indices.data_ptr()), Bi.ctypes.data_as(ctypes.c_void_p), 0,
                    ctypes.byref(hp)) == 0
                self.P.append(hp)
        ops = (ctypes.c_void_p * 3)(*[o.handle for o in self.ops])
        sms = (ctypes.c_void_p * 3)(*self.sm)
        prs = (ctypes.c_void_p * 2)(*self.P)
        self.mg = ctypes.c_void_p()
        assert d.lib.gbpa_multigrid_create(d.ctx, 3, ops, sms, prs, 1e-2, 200, 0, None,
                                           ctypes.byref(self.mg)) == 0

    def close(self):
        lib = self.d.lib
        lib.gbpa_multigrid_destroy(self.mg)
        for h in self.sm[1:]:
            lib.gbpa_chebyshev_destroy(h)
        for h in self.P:
            lib.gbpa_ptransfer_destroy(h)


@pytest.fixture(scope="module")
def g():
    return load_golden("pmg4_p124")


def test_transfer_matches_reference(g):
    from tests.gpu_util import T, H
    H_ = GoldenHierarchy(g)
    lib = H_.d.lib
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    for l in (1, 2):
        k = f"l{l}_"
        x = T(g[k + "P_x"]); y = torch.zeros(g[k + "P_y"].size, dtype=torch.float64, device="cuda")
        assert lib.gbpa_ptransfer_mult(H_.P[l - 1], P(x), P(y)) == 0
        assert rel(H(y), g[k + "P_y"]) < 1e-14
        x = T(g[k + "Pt_x"]); y = torch.zeros(g[k + "Pt_y"].size, dtype=torch.float64, device="cuda")
        assert lib.gbpa_ptransfer_mult_transpose(H_.P[l - 1], P(x), P(y)) == 0
        assert rel(H(y), g[k + "Pt_y"]) < 1e-14
    H_.close()


def test_chebyshev_matches_reference(g):
    from tests.gpu_util import T, H
    H_ = GoldenHierarchy(g)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    for l in (1, 2):
        k = f"l{l}_"
        x = T(g[k + "cheb_x"]); y = torch.zeros_like(x)
        assert H_.d.lib.gbpa_chebyshev_mult(H_.sm[l], P(x), P(y)) == 0
        assert rel(H(y), g[k + "cheb_y"]) < 1e-13
    H_.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_vcycle_and_mg_pcg_match_reference(g, precision):
    """One V-cycle and the MG-preconditioned CG solve with the reference's
    eigenvalue estimates: FP64 and double-float level operators."""
    from mfem_gb300 import _lib
    from tests.gpu_util import T, H
    H_ = GoldenHierarchy(g, precision=precision)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    b = T(g["B_rhs"]); y = torch.zeros_like(b)
    assert H_.d.lib.gbpa_multigrid_mult(H_.mg, P(b), P(y)) == 0
    assert rel(H(y), g["mg_b"]) < 1e-11
    x = torch.zeros_like(b)
    info = _lib.SolveInfo()
    assert H_.d.lib.gbpa_pcg_solve_mg(H_.ops[-1].handle, H_.mg, P(b), P(x), 1e-10, 0.0, 200,
                                      ctypes.byref(info)) == 0
    assert info.converged == 1
    assert abs(info.iterations - int(g["cg_info"][0])) <= 1
    assert rel(H(x), g["X"]) < 1e-10
    H_.close()


def test_power_method_matches_oracle(g):
    """The device power method and the oracle's run the same iteration from
    the same splitmix64 start vector."""
    from tests import oracle_lib
    from tests.test_oracle_mg import levels_from_golden
    H_ = GoldenHierarchy(g)
    o = oracle_lib.load()
    lv = levels_from_golden(g)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    for l in (1, 2):
        h = ctypes.c_void_p()
        assert H_.d.lib.gbpa_chebyshev_create(H_.ops[l].handle, P(H_.diag[l]), 2, 0.0, 10, 1e-8, 12345,
                                              ctypes.byref(h)) == 0
        lam = ctypes.c_double(0.0)
        assert H_.d.lib.gbpa_chebyshev_get_max_eig(h, ctypes.byref(lam)) == 0
        H_.d.lib.gbpa_chebyshev_destroy(h)
        lo = o.power_method(lv[l], 10, 1e-8, 12345)
        assert abs(lam.value - lo) < 1e-10 * lo
    H_.close()


def pmg_problem(n, orders, precision=0, coarse_jacobi=False):
    from mfem_gb300 import fem
    from mfem_gb300.pa import DiffusionMultigrid
    from tests.gpu_util import dev
    dev()
    mesh = fem.CartesianMesh(n, jitter=0.1, seed=1)
    M = DiffusionMultigrid(mesh, orders, "kappa", modes=fem.kappa_modes(3), precision=precision,
                           coarse_jacobi=coarse_jacobi)
    fes = M.spaces[-1]
    b = torch.from_numpy(fem.u01_array(4, fes.ndofs)).cuda()
    b[torch.from_numpy(M.ess[-1]).long().cuda()] = 0.0
    return M, b


@pytest.mark.parametrize("precision,coarse_jacobi", [(0, False), (2, False), (2, True), (1, False), (1, True)])
def test_mg_pcg_solves_the_jacobi_system(precision, coarse_jacobi):
    """On a 10^3 mesh at p=4 (levels 1, 2, 4): the MG-preconditioned solve
    (FP64, double-float or FP32 levels; plain or Jacobi-preconditioned
    coarse CG) reaches the FP64 Jacobi-PCG solution of the same constrained
    system (1e-9) in far fewer iterations."""
    from mfem_gb300 import _lib
    from mfem_gb300.pa import CGSolver, OperatorJacobiSmoother
    from mfem_gb300.pa import PAOperator
    M, b = pmg_problem(10, (1, 2, 4), precision, coarse_jacobi)
    fes, integ = M.spaces[-1], M.integs[-1]
    A = M.operators[-1] if precision != 1 else PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata,
                                                          ess=M.ess[-1])
    x = torch.zeros_like(b)
    cg = CGSolver(); cg.SetRelTol(1e-11); cg.SetMaxIter(500); cg.SetOperator(A); cg.SetPreconditioner(M)
    cg.Mult(b, x)
    assert cg.GetConverged()
    it_mg = cg.GetNumIterations()
    J = OperatorJacobiSmoother(A, M.ess[-1])
    xj = torch.zeros_like(b)
    cj = CGSolver(); cj.SetRelTol(1e-11); cj.SetMaxIter(5000); cj.SetOperator(A); cj.SetPreconditioner(J)
    cj.Mult(b, xj)
    assert cj.GetConverged()
    assert it_mg * 4 < cj.GetNumIterations(), (it_mg, cj.GetNumIterations())
    assert float(torch.linalg.norm(x - xj) / torch.linalg.norm(xj)) < 1e-9


def test_mg_against_oracle_on_own_hierarchy():
    """The library's own hierarchy (maps, tables, qdata from its setup) and
    eigenvalue estimates, run through the oracle's V-cycle solve: same
    solution and iteration count as the device solve."""
    from mfem_gb300 import _lib
    from tests import oracle_lib
    from tests.gpu_util import H
    M, b = pmg_problem(5, (1, 2, 4))
    lv = []
    for l, (fes, integ) in enumerate(zip(M.spaces, M.integs)):
        R = fes.GetElementRestriction()
        diag = None
        lam = 0.0
        Bi = None
        if l > 0:
            diag = H(M.smoothers[l].diag)
            lam = M.smoothers[l].GetMaxEigEstimate()
            Bi = M.prolongations[l - 1].Bi
        lv.append(oracle_lib.mg_level(fes.ne, fes.ndofs, integ.D, integ.Q, H(R.gather_map), H(R.offsets),
                                      H(R.indices), H(integ.B), H(integ.G), H(integ.qdata), M.ess[l],
                                      diag=diag, lam=lam, Bi=Bi))
    o = oracle_lib.load()
    xo, ito, _, convo = o.mg_pcg(lv, H(b), rel_tol=1e-10, max_it=200)
    x = torch.zeros_like(b)
    info = _lib.SolveInfo()
    from tests.gpu_util import dev
    assert dev().lib.gbpa_pcg_solve_mg(M.operators[-1].handle, M.handle, ctypes.c_void_p(b.data_ptr()),
                                       ctypes.c_void_p(x.data_ptr()), 1e-10, 0.0, 200, ctypes.byref(info)) == 0
    assert convo and info.converged == 1
    assert abs(info.iterations - ito) <= 1
    assert rel(H(x), xo) < 1e-10


def test_mg_order_8_hierarchy():
    """Orders 1, 2, 4, 8 (the ex26 doubling to p = 8) on a 4^3 mesh: the
    MG-preconditioned solve reaches the Jacobi-PCG solution."""
    from mfem_gb300.pa import CGSolver, OperatorJacobiSmoother
    M, b = pmg_problem(4, (1, 2, 4, 8), 2)
    A = M.operators[-1]
    x = torch.zeros_like(b)
    cg = CGSolver(); cg.SetRelTol(1e-11); cg.SetMaxIter(500); cg.SetOperator(A); cg.SetPreconditioner(M)
    cg.Mult(b, x)
    assert cg.GetConverged()
    J = OperatorJacobiSmoother(A, M.ess[-1])
    xj = torch.zeros_like(b)
    cj = CGSolver(); cj.SetRelTol(1e-11); cj.SetMaxIter(5000); cj.SetOperator(A); cj.SetPreconditioner(J)
    cj.Mult(b, xj)
    assert cj.GetConverged() and cg.GetNumIterations() * 3 < cj.GetNumIterations()
    assert float(torch.linalg.norm(x - xj) / torch.linalg.norm(xj)) < 1e-9


def test_mg_invalid_arguments_rejected():
    """Mismatched levels and unsupported combinations return
    GBPA_ERR_INVALID_ARGUMENT / GBPA_ERR_UNSUPPORTED without touching the GPU
    state; the context stays usable."""
    from mfem_gb300 import _lib
    from mfem_gb300.pa import PAOperator
    from tests.gpu_util import dev
    d = dev()
    M, b = pmg_problem(3, (1, 2))
    ops, P, S = M.operators, M.prolongations, M.smoothers
    h = ctypes.c_void_p()
    arr = lambda *hs: (ctypes.c_void_p * len(hs))(*hs)
    # smoother of the wrong level
    assert d.lib.gbpa_multigrid_create(d.ctx, 2, arr(ops[0].handle, ops[1].handle), arr(None, None),
                                       arr(P[0].handle), 1e-2, 200, 0, None, ctypes.byref(h)) == -1
    # levels swapped (sizes do not match the transfer)
    assert d.lib.gbpa_multigrid_create(d.ctx, 2, arr(ops[1].handle, ops[0].handle), arr(None, S[1].handle),
                                       arr(P[0].handle), 1e-2, 200, 0, None, ctypes.byref(h)) == -1
    # an FP32 coarse level with a Jacobi coarse solve needs the coarse diagonal
    fes, integ = M.spaces[0], M.integs[0]
    A32 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=M.ess[0], precision=1)
    assert d.lib.gbpa_multigrid_create(d.ctx, 1, arr(A32.handle), None, None, 1e-2, 50, 1, None,
                                       ctypes.byref(h)) == -1
    # the outer CG needs FP64 vectors
    x = torch.zeros_like(b)
    info = _lib.SolveInfo()
    assert d.lib.gbpa_pcg_solve_mg(A32.handle, M.handle, ctypes.c_void_p(b.data_ptr()),
                                   ctypes.c_void_p(x.data_ptr()), 1e-10, 0.0, 10, ctypes.byref(info)) == -1
    # transfer orders beyond p = 9
    assert d.lib.gbpa_ptransfer_create(d.ctx, 1, 2, 8, None, None, None, 11, 1331, None, None, None, None, 0,
                                       ctypes.byref(h)) == -2
    # the hierarchy still works
    y = torch.empty_like(b)
    M.Mult(b, y)
    assert torch.isfinite(y).all()
