"""Batching form: several independent Dirichlet Poisson problems of uneven size
and order solved together (gbpa_batched_pcg_solve*, graph-captured and
persistent schedules) must give the same solutions as solving each problem
alone with gbpa_pcg_solve (which is pinned to the reference's PCG on the
golden cfg1 problem) and as the CPU oracle's PCG: relative L2 <= 1e-10,
iteration counts within 1."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def make_problem(n, p, coeff, seed, ir_points=None):
    from mfem_gb300 import fem
    from mfem_gb300.pa import (DiffusionIntegrator, FiniteElementSpace, OperatorJacobiSmoother,
                               PAOperator)
    mesh = fem.CartesianMesh(n, jitter=0.1, seed=seed)
    fes = FiniteElementSpace(mesh, p)
    integ = DiffusionIntegrator(coeff, ir_points=ir_points)
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    ess = fes.GetBoundaryTrueDofs()
    A = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess)
    M = OperatorJacobiSmoother(A, ess)
    nd = fes.GetNDofs()
    b = torch.from_numpy(fem.u01_array(4 + seed, nd)).cuda()
    b[torch.from_numpy(ess).long().cuda()] = 0.0
    return dict(fes=fes, integ=integ, ess=torch.from_numpy(ess).cuda(), A=A, dinv=M.dinv, b=b,
                x=torch.zeros(nd, dtype=torch.float64, device="cuda"))


def desc(pr):
    from mfem_gb300 import _lib
    R = pr["fes"].GetElementRestriction()
    it = pr["integ"]
    return _lib.ProblemDesc(pr["fes"].ne, pr["fes"].ndofs, it.D, it.Q, it.B.data_ptr(), it.G.data_ptr(),
                            it.qdata.data_ptr(), R.gather_map.data_ptr(), R.offsets.data_ptr(),
                            R.indices.data_ptr(), pr["ess"].data_ptr(), pr["ess"].numel(),
                            pr["dinv"].data_ptr(), pr["b"].data_ptr(), pr["x"].data_ptr())


def test_batched_matches_single_solves():
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    specs = [(3, 2, None), (4, 3, "kappa"), (2, 6, None), (5, 4, "kappa"), (3, 5, 2.5), (6, 2, "kappa")]
    probs = [make_problem(n, p, c, s) for s, (n, p, c) in enumerate(specs)]
    arr = (_lib.ProblemDesc * len(probs))(*[desc(pr) for pr in probs])
    its = (ctypes.c_int * len(probs))()
    conv = (ctypes.c_int * len(probs))()
    norms = (ctypes.c_double * len(probs))()
    secs = ctypes.c_double(0)
    st = d.lib.gbpa_batched_pcg_solve(d.ctx, len(probs), arr, 1e-10, 0.0, 1000, its, conv, norms,
                                      ctypes.byref(secs))
    assert st == 0
    for k, pr in enumerate(probs):
        X = torch.zeros_like(pr["x"])
        info = _lib.SolveInfo()
        st = d.lib.gbpa_pcg_solve(pr["A"].handle, ctypes.c_void_p(pr["dinv"].data_ptr()),
                                  ctypes.c_void_p(pr["b"].data_ptr()), ctypes.c_void_p(X.data_ptr()),
                                  1e-10, 0.0, 1000, 0, ctypes.byref(info))
        assert st == 0 and info.converged == 1
        assert conv[k] == 1
        assert abs(its[k] - info.iterations) <= 1, (k, its[k], info.iterations)
        err = float(torch.linalg.norm(pr["x"] - X) / torch.linalg.norm(X))
        assert err < 1e-10, (k, err)


def test_batched_against_oracle():
    from mfem_gb300 import _lib
    from tests import oracle_lib
    from tests.gpu_util import dev
    d = dev()
    pr = make_problem(4, 3, "kappa", 11)
    arr = (_lib.ProblemDesc * 1)(desc(pr))
    its = (ctypes.c_int * 1)()
    conv = (ctypes.c_int * 1)()
    st = d.lib.gbpa_batched_pcg_solve(d.ctx, 1, arr, 1e-10, 0.0, 1000, its, conv, None, None)
    assert st == 0 and conv[0] == 1
    o = oracle_lib.load()
    R = pr["fes"].GetElementRestriction()
    it = pr["integ"]
    Xo, ito, _, convo = o.pcg_diffusion(pr["fes"].ne, pr["fes"].ndofs, True, it.D, it.Q,
                                        R.gather_map.cpu().numpy(), R.offsets.cpu().numpy(),
                                        R.indices.cpu().numpy(), it.B.cpu().numpy(), it.G.cpu().numpy(),
                                        it.qdata.cpu().numpy(), pr["ess"].cpu().numpy(),
                                        pr["dinv"].cpu().numpy(), pr["b"].cpu().numpy(),
                                        rel_tol=1e-10, max_it=1000)
    assert convo and abs(ito - its[0]) <= 1
    x = pr["x"].cpu().numpy()
    assert np.linalg.norm(x - Xo) / np.linalg.norm(Xo) < 1e-10


def solve_ex(d, probs, precision, schedule, rel_tol=1e-10, max_it=1000):
    from mfem_gb300 import _lib
    arr = (_lib.ProblemDesc * len(probs))(*[desc(pr) for pr in probs])
    its = (ctypes.c_int * len(probs))()
    conv = (ctypes.c_int * len(probs))()
    st = d.lib.gbpa_batched_pcg_solve_ex(d.ctx, len(probs), arr, precision, schedule, rel_tol, 0.0, max_it,
                                         its, conv, None, None)
    return st, list(its), list(conv)


def single_solve(d, pr):
    from mfem_gb300 import _lib
    X = torch.zeros_like(pr["x"])
    info = _lib.SolveInfo()
    assert d.lib.gbpa_pcg_solve(pr["A"].handle, ctypes.c_void_p(pr["dinv"].data_ptr()),
                                ctypes.c_void_p(pr["b"].data_ptr()), ctypes.c_void_p(X.data_ptr()),
                                1e-10, 0.0, 1000, 0, ctypes.byref(info)) == 0
    return X, info.iterations


def test_batched_rejects_unsupported_order():
    """The persistent schedule's runtime-size kernel stops at p = 6; the graph
    schedule stops at d1d, q1d <= 10."""
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    pr = make_problem(2, 7, None, 1)
    st, _, _ = solve_ex(d, [pr], _lib.GBPA_F64, _lib.GBPA_BATCH_PERSISTENT, max_it=100)
    assert st == -2
    pr10 = make_problem(1, 10, None, 1)   # d1d = 11
    st, _, _ = solve_ex(d, [pr10], _lib.GBPA_F64, _lib.GBPA_BATCH_GRAPH, max_it=100)
    assert st == -2


def test_batched_schedules_agree():
    """Graph and persistent schedules run the same iteration: same iteration
    counts (within 1) and solutions within 1e-12 of each other, FP64 and
    double-float."""
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    specs = [(3, 2, None), (5, 3, "kappa"), (2, 6, "kappa"), (4, 4, 1.5), (7, 2, "kappa")]
    probs = [make_problem(n, p, c, 20 + s) for s, (n, p, c) in enumerate(specs)]
    for prec in (_lib.GBPA_F64, _lib.GBPA_F64X2):
        st, its_p, conv_p = solve_ex(d, probs, prec, _lib.GBPA_BATCH_PERSISTENT)
        assert st == 0 and all(conv_p)
        xs_p = [pr["x"].clone() for pr in probs]
        st, its_g, conv_g = solve_ex(d, probs, prec, _lib.GBPA_BATCH_GRAPH)
        assert st == 0 and all(conv_g)
        for k, pr in enumerate(probs):
            assert abs(its_p[k] - its_g[k]) <= 1, (prec, k, its_p[k], its_g[k])
            err = float(torch.linalg.norm(pr["x"] - xs_p[k]) / torch.linalg.norm(xs_p[k]))
            assert err < 1e-12, (prec, k, err)


def test_batched_graph_high_order_and_compaction():
    """Graph schedule with orders the persistent kernel does not cover (p = 7,
    8 and p = 9 with q1d = 10, all through the runtime-size kernel) next to
    compile-time ones, and iteration counts spread widely, so the work tables
    are rebuilt as problems converge; every problem matches its
    single-problem solve."""
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    specs = [(1, 2, None, None), (2, 7, "kappa", None), (6, 2, "kappa", None), (1, 9, None, 10),
             (2, 8, 3.0, None), (8, 3, "kappa", None)]
    probs = [make_problem(n, p, c, 40 + s, q) for s, (n, p, c, q) in enumerate(specs)]
    st, its, conv = solve_ex(d, probs, _lib.GBPA_F64, _lib.GBPA_BATCH_GRAPH)
    assert st == 0 and all(conv)
    assert max(its) > 3 * min(its)
    for k, pr in enumerate(probs):
        X, it1 = single_solve(d, pr)
        assert abs(its[k] - it1) <= 1, (k, its[k], it1)
        err = float(torch.linalg.norm(pr["x"] - X) / torch.linalg.norm(X))
        assert err < 1e-10, (k, err)


def test_batched_zero_rhs_and_empty_problem():
    """A problem whose right-hand side is zero converges at iteration 0 with
    x = 0 (the stopping rule nom <= max(rel_tol^2 nom, abs_tol^2) holds with
    nom = 0), and so does a problem with no dofs; the others are unaffected."""
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    probs = [make_problem(3, 2, None, 60), make_problem(3, 3, "kappa", 61)]
    probs[0]["b"].zero_()
    probs[0]["x"].fill_(7.0)
    for schedule in (_lib.GBPA_BATCH_GRAPH, _lib.GBPA_BATCH_PERSISTENT):
        descs = [desc(pr) for pr in probs]
        empty = _lib.ProblemDesc(0, 0, 3, 4, None, None, None, None, None, None, None, 0, None, None, None)
        arr = (_lib.ProblemDesc * 3)(descs[0], empty, descs[1])
        its = (ctypes.c_int * 3)()
        conv = (ctypes.c_int * 3)()
        st = d.lib.gbpa_batched_pcg_solve_ex(d.ctx, 3, arr, _lib.GBPA_F64, schedule, 1e-10, 0.0, 1000, its,
                                             conv, None, None)
        assert st == 0
        assert list(conv) == [1, 1, 1] and its[0] == 0 and its[1] == 0 and its[2] > 0
        assert float(probs[0]["x"].abs().max()) == 0.0
        X, _ = single_solve(d, probs[1])
        assert float(torch.linalg.norm(probs[1]["x"] - X) / torch.linalg.norm(X)) < 1e-10


def test_batched_double_float_matches_single_solves():
    """GBPA_F64X2 arithmetic in the persistent batched solve reaches the same
    solutions as the single-problem FP64 PCG (1e-10)."""
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    specs = [(3, 2, None), (4, 4, "kappa"), (2, 6, "kappa")]
    probs = [make_problem(n, p, c, s) for s, (n, p, c) in enumerate(specs)]
    arr = (_lib.ProblemDesc * len(probs))(*[desc(pr) for pr in probs])
    conv = (ctypes.c_int * len(probs))()
    st = d.lib.gbpa_batched_pcg_solve_precision(d.ctx, len(probs), arr, 2, 1e-10, 0.0, 1000, None, conv,
                                                None, None)
    assert st == 0 and all(conv[k] == 1 for k in range(len(probs)))
    for pr in probs:
        X = torch.zeros_like(pr["x"])
        info = _lib.SolveInfo()
        assert d.lib.gbpa_pcg_solve(pr["A"].handle, ctypes.c_void_p(pr["dinv"].data_ptr()),
                                    ctypes.c_void_p(pr["b"].data_ptr()), ctypes.c_void_p(X.data_ptr()),
                                    1e-10, 0.0, 1000, 0, ctypes.byref(info)) == 0
        assert float(torch.linalg.norm(pr["x"] - X) / torch.linalg.norm(X)) < 1e-9
