"""The tensor-core layout of the FP32 diffusion operator (GBPA_LAYOUT_TC: the
element contraction as two Kronecker GEMMs per tile of 128 elements on
tcgen05, fp16 hi/lo operand limbs, FP32 accumulation). Checked against the
reference's own apply on the golden cases (the FP32 bar, 1e-5 relative L2),
against the CUDA-core FP32 kernel, on constrained and atomic-scatter
operators, on element counts that leave a partial last tile, on inputs whose
magnitudes span many binades (the per-element power-of-two scaling), and
inside the mixed-precision solve."""
import numpy as np
import pytest
import torch

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu

TC = 2
# golden cases with symmetric qdata and a (D, Q) pair the tensor-core kernel covers
CASES = ["cart2_p2_one", "jit3_p3_fn", "jit2_p4_sym", "jit2_p4_vec", "curv2_p3_fn"]


class tc_layout:
    """Select the tensor-core layout for FP32 diffusion at (D, Q) while the
    block runs; restore the previous layout afterwards."""

    def __init__(self, lib, D, Q, layout=TC):
        self.lib, self.D, self.Q, self.layout = lib, D, Q, layout

    def __enter__(self):
        import ctypes
        n = ctypes.c_int(0)
        self.prev = self.lib.gbpa_get_apply_layout(0, 1, self.D, self.Q, ctypes.byref(n))
        self.prev_nbz = n.value
        assert self.lib.gbpa_set_apply_layout(0, 1, self.D, self.Q, self.layout, 0) == 0
        return self

    def __exit__(self, *a):
        self.lib.gbpa_set_apply_layout(0, 1, self.D, self.Q, self.prev, self.prev_nbz)


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("case", CASES)
def test_tc_apply_matches_reference(case):
    from mfem_gb300.pa import ElementRestriction, PAOperator
    from tests.gpu_util import T, H, dev
    d = dev()
    g = load_golden(case)
    ne, ndofs, D, Q = (int(v) for v in g["meta"][:4])
    R = ElementRestriction.from_maps(ne, D ** 3, ndofs, g["gather_map"], g["offsets"], g["indices"])
    B, G, qd = T(g["B"]), T(g["G"]), T(g["qdata_diff"])
    x = T(g["x"]).float()
    slab = PAOperator(0, R, D, Q, B, G, qd, precision=1)
    y_slab = torch.empty_like(x)
    slab.Mult(x, y_slab)
    with tc_layout(d.lib, D, Q):
        op = PAOperator(0, R, D, Q, B, G, qd, precision=1)
        y = torch.empty_like(x)
        op.Mult(x, y)
        torch.cuda.synchronize()
    assert _rel(H(y), g["y_diff"]) < 1e-5
    assert _rel(H(y), H(y_slab).astype(np.float64)) < 5e-6   # two FP32 results, each ~1e-6 from FP64


@pytest.mark.parametrize("p,n", [(4, 7), (4, 12), (3, 9), (2, 13)])
def test_tc_apply_against_oracle_partial_tiles(oracle, p, n):
    """Jittered meshes whose element counts (343, 1728, 729, 2197) leave a
    partial last tile of 128; L->L against the FP64 oracle and against the
    CUDA-core FP32 kernel."""
    from mfem_gb300 import fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, PAOperator
    from tests.gpu_util import H, dev
    d = dev()
    fes = FiniteElementSpace(fem.CartesianMesh(n, jitter=0.1, seed=2), p)
    integ = DiffusionIntegrator()
    integ.AssemblePA(fes)
    R = fes.GetElementRestriction()
    x64 = torch.from_numpy(2 * fem.u01_array(9, fes.ndofs) - 1).cuda()
    x = x64.float()
    yo = oracle.pa_mult(0, fes.ne, fes.ndofs, True, integ.D, integ.Q, R.gather_map.cpu().numpy(),
                        R.offsets.cpu().numpy(), R.indices.cpu().numpy(), integ.B.cpu().numpy(),
                        integ.G.cpu().numpy(), integ.qdata.cpu().numpy(), x64.cpu().numpy())
    slab = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, precision=1)
    ys = torch.empty_like(x)
    slab.Mult(x, ys)
    with tc_layout(d.lib, integ.D, integ.Q):
        for scatter in (0, 1):
            op = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, precision=1, scatter=scatter)
            y = torch.empty_like(x)
            op.Mult(x, y)
            torch.cuda.synchronize()
            assert _rel(H(y), yo) < 1e-5
            assert _rel(H(y), H(ys).astype(np.float64)) < 5e-6


def test_tc_wide_dynamic_range_and_constrained(oracle):
    """x whose magnitude grows smoothly from 2^-30 to 2^30 across the mesh
    (the per-element power-of-two scaling keeps every region's accuracy:
    within each magnitude band the tensor-core result meets the FP32 bar,
    1e-5 relative L2, as the CUDA-core FP32 kernel does), on a constrained
    operator (y[ess] = x[ess])."""
    from mfem_gb300 import fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, PAOperator
    from tests.gpu_util import H, dev
    d = dev()
    n, p = 8, 4
    fes = FiniteElementSpace(fem.CartesianMesh(n, jitter=0.1, seed=4), p)
    integ = DiffusionIntegrator()
    integ.AssemblePA(fes)
    R = fes.GetElementRestriction()
    rng = np.random.default_rng(3)
    N = p * n + 1
    idx = np.arange(fes.ndofs)
    i, j = idx % N, (idx // N) % N
    t = (i + j) / (2.0 * (N - 1))
    xh = rng.uniform(-1, 1, fes.ndofs) * 2.0 ** (60.0 * t - 30.0)
    x = torch.from_numpy(xh).cuda().float()
    ess = fes.GetBoundaryTrueDofs()
    gm, off, ind = R.gather_map.cpu().numpy(), R.offsets.cpu().numpy(), R.indices.cpu().numpy()
    z = x.double().cpu().numpy().copy()
    z[ess] = 0.0
    yo = oracle.pa_mult(0, fes.ne, fes.ndofs, True, integ.D, integ.Q, gm, off, ind, integ.B.cpu().numpy(),
                        integ.G.cpu().numpy(), integ.qdata.cpu().numpy(), z)
    yo[ess] = x.double().cpu().numpy()[ess]
    slab = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess, precision=1)
    ys = torch.empty_like(x)
    slab.Mult(x, ys)
    with tc_layout(d.lib, integ.D, integ.Q):
        op = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess, precision=1)
        y = torch.empty_like(x)
        op.Mult(x, y)
        torch.cuda.synchronize()
    yh, ysh = H(y).astype(np.float64), H(ys).astype(np.float64)
    assert np.all(np.isfinite(yh))
    band = np.minimum((t * 6).astype(int), 5)
    for b in range(6):
        m = band == b
        e_tc, e_slab = _rel(yh[m], yo[m]), _rel(ysh[m], yo[m])
        assert e_tc < 1e-5 and e_slab < 1e-5, (b, e_tc, e_slab)


def test_tc_mixed_precision_solve():
    """The reliable-update precision form with the tensor-core FP32 inner
    operator reaches the same FP64 solution as with the CUDA-core one."""
    import ctypes
    from mfem_gb300 import _lib, fem
    from mfem_gb300.pa import (DiffusionIntegrator, FiniteElementSpace, OperatorJacobiSmoother, PAOperator)
    from tests.gpu_util import dev
    d = dev()
    fes = FiniteElementSpace(fem.CartesianMesh(8, jitter=0.1, seed=1), 4)
    integ = DiffusionIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    ess = fes.GetBoundaryTrueDofs()
    A64 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess)
    M = OperatorJacobiSmoother(A64, ess)
    b = torch.from_numpy(fem.u01_array(4, fes.ndofs)).cuda()
    b[torch.from_numpy(ess).long().cuda()] = 0.0
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    info = _lib.SolveInfo()
    X64 = torch.zeros_like(b)
    assert d.lib.gbpa_pcg_solve(A64.handle, P(M.dinv), P(b), P(X64), 1e-12, 0.0, 5000, 0, ctypes.byref(info)) == 0
    d32 = M.dinv.float()
    with tc_layout(d.lib, integ.D, integ.Q):
        A32 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess, precision=1)
        Xr = torch.zeros_like(b)
        st = d.lib.gbpa_pcg_solve_mixed_reliable(A64.handle, A32.handle, P(d32), P(b), P(Xr), 1e-10, 0.1, 5000,
                                                 ctypes.byref(info))
    assert st == 0 and info.converged
    assert info.true_rel_residual <= 1e-10
    assert float(torch.linalg.norm(Xr - X64) / torch.linalg.norm(X64)) < 1e-9


def test_tc_layout_api():
    from tests.gpu_util import dev
    d = dev()
    lib = d.lib
    assert lib.gbpa_set_apply_layout(0, 0, 5, 6, TC, 0) == -2      # FP64: no tensor-core kernel
    assert lib.gbpa_set_apply_layout(1, 1, 5, 6, TC, 0) == -2      # mass
    assert lib.gbpa_set_apply_layout(0, 1, 7, 8, TC, 0) == -2      # order without a kernel
    with tc_layout(lib, 5, 6):
        assert lib.gbpa_get_apply_layout(0, 1, 5, 6, None) == TC
