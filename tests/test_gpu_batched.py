"""Batching form: several independent Dirichlet Poisson problems of uneven size
and order solved in one persistent launch (gbpa_batched_pcg_solve) must give
the same solutions as solving each problem alone with gbpa_pcg_solve (which is
pinned to the reference's PCG on the golden cfg1 problem) and as the CPU
oracle's PCG: relative L2 <= 1e-10, iteration counts within 1."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def make_problem(n, p, coeff, seed):
    from mfem_gb300 import fem
    from mfem_gb300.pa import (DiffusionIntegrator, FiniteElementSpace, OperatorJacobiSmoother,
                               PAOperator)
    mesh = fem.CartesianMesh(n, jitter=0.1, seed=seed)
    fes = FiniteElementSpace(mesh, p)
    integ = DiffusionIntegrator(coeff)
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


def test_batched_rejects_unsupported_order():
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    pr = make_problem(2, 7, None, 1)     # p = 7 exceeds the batched kernel's p <= 6
    arr = (_lib.ProblemDesc * 1)(desc(pr))
    st = d.lib.gbpa_batched_pcg_solve(d.ctx, 1, arr, 1e-10, 0.0, 100, None, None, None, None)
    assert st == -2


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
