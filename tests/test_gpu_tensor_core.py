"""The tensor-core layout of the FP32 diffusion operator (GBPA_LAYOUT_TC: the
element contraction as two Kronecker GEMMs per tile of 128 elements on
tcgen05, fp16 hi/lo operand limbs, FP32 accumulation). Checked against the
reference's own apply on the golden cases (the FP32 bar, 1e-5 relative L2),
against the CUDA-core FP32 kernel, on constrained and atomic-scatter
operators, on element counts that leave a partial last tile, on inputs whose
magnitudes span many binades (the per-element power-of-two scaling), and
inside the mixed-precision solve. The block form (tiles of 16 elements x 8
interleaved right-hand sides) is checked column by column against the FP64
apply and the CUDA-core block kernel."""
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


# ----------------------------------------------------------------- block form
class block_layout:
    """Select the FP32 block apply's kernel for (D, Q, nrhs) while the block
    runs; restore the previous choice afterwards."""

    def __init__(self, lib, D, Q, R, layout):
        self.lib, self.D, self.Q, self.R, self.layout = lib, D, Q, R, layout

    def __enter__(self):
        self.prev = self.lib.gbpa_get_block_apply_layout(self.D, self.Q, self.R)
        assert self.lib.gbpa_set_block_apply_layout(self.D, self.Q, self.R, self.layout) == 0
        return self

    def __exit__(self, *a):
        self.lib.gbpa_set_block_apply_layout(self.D, self.Q, self.R, self.prev)


def _block_ops(n, p, curved):
    from mfem_gb300 import fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, PAOperator
    mesh = fem.CartesianMesh(n, jitter=0.0 if curved else 0.1, seed=3, curved=curved)
    fes = FiniteElementSpace(mesh, p)
    integ = DiffusionIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(5))
    ess = fes.GetBoundaryTrueDofs()
    A64 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess)
    A32 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess, precision=1)
    return fes, integ, A64, A32


def _mult_block(lib, op, R, X, Y):
    import ctypes
    return lib.gbpa_operator_mult_block(op.handle, R, ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(Y.data_ptr()))


@pytest.mark.parametrize("p,n,curved", [(5, 5, True), (5, 7, False), (4, 9, False)])
def test_tc_block_apply_against_fp64_and_cuda_core(p, n, curved):
    """The tensor-core block apply (tiles of 16 elements x 8 interleaved
    right-hand sides; 125, 343 and 729 elements leave a partial last tile) on
    a constrained lognormal-kappa operator: every column against the FP64
    single apply (the FP32 bar, 1e-5 relative L2) and against the CUDA-core
    block kernel (two FP32 results, 5e-6)."""
    from tests.gpu_util import dev
    d = dev()
    fes, integ, A64, A32 = _block_ops(n, p, curved)
    D, Q, R, nd = integ.D, integ.Q, 8, fes.ndofs
    assert d.lib.gbpa_get_block_apply_layout(D, Q, R) == TC
    gen = torch.Generator(device="cuda").manual_seed(21)
    X64 = (torch.rand(nd, R, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1).contiguous()
    X32 = X64.float().contiguous()
    Y = torch.full_like(X32, float("nan"))
    assert _mult_block(d.lib, A32, R, X32, Y) == 0
    with block_layout(d.lib, D, Q, R, 0):
        Yc = torch.full_like(X32, float("nan"))
        assert _mult_block(d.lib, A32, R, X32, Yc) == 0
    torch.cuda.synchronize()
    assert d.error_flags() == 0
    for r in range(R):
        y64 = torch.empty(nd, dtype=torch.float64, device="cuda")
        A64.Mult(X64[:, r].contiguous(), y64)
        yr = Y[:, r].double()
        assert float(torch.linalg.norm(yr - y64) / torch.linalg.norm(y64)) < 1e-5, r
        assert float(torch.linalg.norm(yr - Yc[:, r].double()) / torch.linalg.norm(y64)) < 5e-6, r


def test_tc_block_apply_wide_dynamic_range():
    """Right-hand side r scaled by 2^(8 r - 28), each varying smoothly over
    2^-10..2^10 across the mesh: per-row scaling keeps every column at the
    FP32 bar (1e-5 relative L2 against the FP64 apply)."""
    from tests.gpu_util import dev
    d = dev()
    fes, integ, A64, A32 = _block_ops(6, 5, False)
    nd, R = fes.ndofs, 8
    t = torch.linspace(0, 1, nd, dtype=torch.float64, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(22)
    X64 = torch.empty(nd, R, dtype=torch.float64, device="cuda")
    for r in range(R):
        u = torch.rand(nd, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
        X64[:, r] = u * torch.pow(2.0, 20.0 * t - 10.0) * 2.0 ** (8 * r - 28)
    X32 = X64.float().contiguous()
    X64 = X32.double().contiguous()
    Y = torch.empty_like(X32)
    assert _mult_block(d.lib, A32, R, X32, Y) == 0
    torch.cuda.synchronize()
    assert bool(torch.isfinite(Y).all())
    for r in range(R):
        y64 = torch.empty(nd, dtype=torch.float64, device="cuda")
        A64.Mult(X64[:, r].contiguous(), y64)
        assert float(torch.linalg.norm(Y[:, r].double() - y64) / torch.linalg.norm(y64)) < 1e-5, r


def test_tc_block_layout_api():
    from tests.gpu_util import dev
    lib = dev().lib
    assert lib.gbpa_get_block_apply_layout(6, 7, 8) == TC
    assert lib.gbpa_get_block_apply_layout(5, 6, 8) == TC
    assert lib.gbpa_get_block_apply_layout(4, 5, 8) == 0          # no tensor-core block kernel
    assert lib.gbpa_get_block_apply_layout(6, 7, 4) == 0
    assert lib.gbpa_set_block_apply_layout(4, 5, 8, TC) == -2
    assert lib.gbpa_set_block_apply_layout(6, 7, 8, 1) == -1       # the 3D layout has no block kernel
    assert lib.gbpa_set_block_apply_layout(0, 7, 8, 0) == -1
    with block_layout(lib, 6, 7, 8, 0):
        assert lib.gbpa_get_block_apply_layout(6, 7, 8) == 0
    assert lib.gbpa_get_block_apply_layout(6, 7, 8) == TC
