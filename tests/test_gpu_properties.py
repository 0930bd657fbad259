"""Size-independent properties at larger sizes than the golden cases, edge
cases the reference handles, and failure reporting without any GPU fault
(poisoned inputs on the host; the library must return a status and the
context must stay usable)."""
import ctypes
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def setup(n, p, coeff=None, kind="diffusion", jitter=0.1, q=None):
    from mfem_gb300 import fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, MassIntegrator, PAOperator
    from tests.gpu_util import dev
    dev()
    mesh = fem.CartesianMesh(n, jitter=jitter, seed=1)
    fes = FiniteElementSpace(mesh, p)
    integ = (DiffusionIntegrator if kind == "diffusion" else MassIntegrator)(coeff, ir_points=q)
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    op = PAOperator(0 if kind == "diffusion" else 1, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata)
    return fes, integ, op


@pytest.mark.parametrize("p", [1, 2, 4, 6, 8])
def test_diffusion_annihilates_constants(p):
    """A 1 = 0 for the (unconstrained) diffusion operator on any mesh."""
    fes, integ, op = setup(10 if p < 6 else 5, p, "kappa")
    one = torch.ones(fes.ndofs, dtype=torch.float64, device="cuda")
    y = torch.empty_like(one)
    op.Mult(one, y)
    x = torch.rand_like(one)
    ax = torch.empty_like(one)
    op.Mult(x, ax)
    assert float(y.abs().max()) < 1e-12 * float(ax.abs().max())


@pytest.mark.parametrize("p", [1, 3, 5])
def test_mass_of_ones_is_volume(p):
    """1^T M 1 = |Omega| = 1 for the unit cube (jitter keeps the volume)."""
    fes, integ, op = setup(9, p, None, kind="mass")
    one = torch.ones(fes.ndofs, dtype=torch.float64, device="cuda")
    y = torch.empty_like(one)
    op.Mult(one, y)
    assert abs(float(y.sum()) - 1.0) < 1e-12


def test_linear_functions_interior_zero_affine():
    """On an affine mesh the diffusion apply of a linear function vanishes at
    interior dofs (the exact solution of the Laplace problem)."""
    from mfem_gb300 import fem
    fes, integ, op = setup(6, 3, None, jitter=0.0)
    sp = fes.space
    N1 = sp.N1
    g = np.zeros((N1, N1, N1, 3))
    pts = []
    nodes = fem.gauss_lobatto(4)
    coords = np.concatenate([[(e + nodes[:-1]) / 6 for e in range(6)]]).ravel()
    coords = np.append(coords, 1.0)
    iz, iy, ix = np.meshgrid(coords, coords, coords, indexing="ij")
    f = (1.0 + 2.0 * ix - 3.0 * iy + 0.5 * iz).ravel()
    x = torch.from_numpy(f).cuda()
    y = torch.empty_like(x)
    op.Mult(x, y)
    interior = np.setdiff1d(np.arange(fes.ndofs), fes.GetBoundaryTrueDofs())
    yi = y.cpu().numpy()[interior]
    assert np.abs(yi).max() < 1e-11


@pytest.mark.parametrize("prec", [0, 2])
def test_symmetry_and_linearity(prec):
    from mfem_gb300.pa import PAOperator
    fes, integ, op = setup(8, 4, "kappa")
    if prec:
        op = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, precision=prec)
    n = fes.ndofs
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    z = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    ax, az, axz = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    op.Mult(x, ax); op.Mult(z, az); op.Mult(2.0 * x - 3.0 * z, axz)
    assert float(torch.linalg.norm(axz - (2 * ax - 3 * az)) / torch.linalg.norm(axz)) < 1e-13
    assert abs(float(torch.dot(z, ax) - torch.dot(x, az))) < 1e-12 * abs(float(torch.dot(x, ax)))


def test_large_apply_matches_oracle():
    """p=4 on 20^3 elements (~0.5 M DOFs): FP64 and double-float L->L applies
    against the CPU oracle on the same maps and qdata."""
    from mfem_gb300.pa import PAOperator
    from tests import oracle_lib
    fes, integ, op = setup(20, 4, "kappa")
    R = fes.GetElementRestriction()
    x = torch.rand(fes.ndofs, dtype=torch.float64, device="cuda") - 0.5
    y = torch.empty_like(x)
    op.Mult(x, y)
    o = oracle_lib.load()
    yo = o.pa_mult(0, fes.ne, fes.ndofs, True, integ.D, integ.Q, R.gather_map.cpu().numpy(),
                   R.offsets.cpu().numpy(), R.indices.cpu().numpy(), integ.B.cpu().numpy(),
                   integ.G.cpu().numpy(), integ.qdata.cpu().numpy(), x.cpu().numpy())
    assert np.linalg.norm(y.cpu().numpy() - yo) / np.linalg.norm(yo) < 1e-12
    opx = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, precision=2)
    opx.Mult(x, y)
    assert np.linalg.norm(y.cpu().numpy() - yo) / np.linalg.norm(yo) < 1e-12


@pytest.mark.parametrize("p", [4, 5])
def test_reduced_precision_constrained_apply(p):
    """FP32 and double-float constrained L->L applies (pre-masked gather map;
    FP32 qdata staged by bulk copies, at p=5 with odd Q where the last
    block's aligned copy would pass the end of the array and the block reads
    global memory) against the FP64 constrained apply."""
    from mfem_gb300.pa import PAOperator
    fes, integ, _ = setup(16 if p == 4 else 13, p, "kappa")
    ess = fes.GetBoundaryTrueDofs()
    args = (0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata)
    op64 = PAOperator(*args, ess=ess)
    x = torch.rand(fes.ndofs, dtype=torch.float64, device="cuda") - 0.5
    y64 = torch.empty_like(x)
    op64.Mult(x, y64)
    opx = PAOperator(*args, ess=ess, precision=2)
    yx = torch.empty_like(x)
    opx.Mult(x, yx)
    assert float(torch.linalg.norm(yx - y64) / torch.linalg.norm(y64)) < 1e-12
    op32 = PAOperator(*args, ess=ess, precision=1)
    x32 = x.float()
    y32 = torch.empty_like(x32)
    op32.Mult(x32, y32)
    assert float(torch.linalg.norm(y32.double() - y64) / torch.linalg.norm(y64)) < 1e-5


def test_under_integration_d_greater_than_q():
    """D > Q (p=4 with a 3-point rule) runs through the generic apply kernel."""
    from tests import oracle_lib
    fes, integ, op = setup(3, 4, None, q=3)
    R = fes.GetElementRestriction()
    x = torch.rand(fes.ndofs, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    op.Mult(x, y)
    o = oracle_lib.load()
    yo = o.pa_mult(0, fes.ne, fes.ndofs, True, integ.D, integ.Q, R.gather_map.cpu().numpy(),
                   R.offsets.cpu().numpy(), R.indices.cpu().numpy(), integ.B.cpu().numpy(),
                   integ.G.cpu().numpy(), integ.qdata.cpu().numpy(), x.cpu().numpy())
    assert np.linalg.norm(y.cpu().numpy() - yo) / np.linalg.norm(yo) < 1e-12


def test_empty_inputs():
    from tests.gpu_util import dev, p
    d = dev()
    assert d.lib.gbpa_diffusion_apply3d(d.ctx, 0, 1, 3, 4, None, None, None, None, None, None, None) == 0
    assert d.lib.gbpa_restriction_mult(d.ctx, 0, 8, 1, 0, 0, None, None, None) == 0
    r = ctypes.c_double(1.0)
    assert d.lib.gbpa_vec_dot(d.ctx, 0, None, None, ctypes.byref(r)) == 0 and r.value == 0.0


def test_vdim3_restriction_matches_scalar():
    """vdim = 3 restriction (byNODES and byVDIM) equals three scalar gathers."""
    from tests.gpu_util import dev, p
    d = dev()
    fes, integ, op = setup(3, 2, None)
    R = fes.GetElementRestriction()
    n, nd, ne = fes.ndofs, 27, fes.ne
    for byvdim in (0, 1):
        x = torch.rand(3 * n, dtype=torch.float64, device="cuda")
        xc = x.view(n, 3).t().contiguous() if byvdim else x.view(3, n)
        y = torch.empty(nd * 3 * ne, dtype=torch.float64, device="cuda")
        assert d.lib.gbpa_restriction_mult(d.ctx, ne, nd, 3, byvdim, n, p(R.gather_map), p(x), p(y)) == 0
        yv = y.view(ne, 3, nd)
        for c in range(3):
            ys = torch.empty(nd * ne, dtype=torch.float64, device="cuda")
            R.Mult(xc[c].contiguous(), ys)
            assert torch.equal(yv[:, c, :].reshape(-1), ys)
        back = torch.empty(3 * n, dtype=torch.float64, device="cuda")
        assert d.lib.gbpa_restriction_mult_transpose(d.ctx, ne, nd, 3, byvdim, n, p(R.offsets),
                                                     p(R.indices), p(y), p(back), 0) == 0
        bc = back.view(n, 3).t() if byvdim else back.view(3, n)
        for c in range(3):
            ys = torch.empty(n, dtype=torch.float64, device="cuda")
            R.MultTranspose(yv[:, c, :].contiguous().view(-1), ys)
            assert torch.equal(bc[c].contiguous(), ys)


# ------------------------------------------------------------- failure paths
def test_zero_diagonal_reported_and_context_usable():
    from tests.gpu_util import dev, p
    d = dev()
    diag = torch.ones(100, dtype=torch.float64, device="cuda")
    diag[17] = 0.0
    dinv = torch.empty_like(diag)
    assert d.lib.gbpa_jacobi_setup(d.ctx, 100, p(diag), None, 0, 1.0, p(dinv)) == -5
    diag[17] = 2.0
    assert d.lib.gbpa_jacobi_setup(d.ctx, 100, p(diag), None, 0, 1.0, p(dinv)) == 0
    assert float(dinv[17]) == 0.5


def test_nan_input_to_pcg_reported():
    from mfem_gb300 import _lib
    from mfem_gb300.pa import OperatorJacobiSmoother, PAOperator
    from tests.gpu_util import dev, p
    d = dev()
    fes, integ, _ = setup(4, 2, None)
    ess = fes.GetBoundaryTrueDofs()
    A = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess)
    M = OperatorJacobiSmoother(A, ess)
    b = torch.ones(fes.ndofs, dtype=torch.float64, device="cuda")
    b[5] = float("nan")
    x = torch.zeros_like(b)
    info = _lib.SolveInfo()
    st = d.lib.gbpa_pcg_solve(A.handle, p(M.dinv), p(b), p(x), 1e-10, 0.0, 100, 0, ctypes.byref(info))
    assert st == -4
    b[5] = 1.0
    b[torch.from_numpy(ess).long().cuda()] = 0.0
    st = d.lib.gbpa_pcg_solve(A.handle, p(M.dinv), p(b), p(x), 1e-10, 0.0, 500, 0, ctypes.byref(info))
    assert st == 0 and info.converged == 1


def test_out_of_range_ess_rejected():
    from mfem_gb300 import _lib
    from tests.gpu_util import dev
    d = dev()
    fes, integ, _ = setup(2, 2, None)
    R = fes.GetElementRestriction()
    bad = torch.tensor([0, 1, fes.ndofs + 5], dtype=torch.int32, device="cuda")
    desc = _lib.OperatorDesc(0, 0, fes.ne, fes.ndofs, integ.D, integ.Q, 1, integ.B.data_ptr(),
                             integ.G.data_ptr(), integ.qdata.data_ptr(), R.gather_map.data_ptr(),
                             R.offsets.data_ptr(), R.indices.data_ptr(), bad.data_ptr(), 3, 0)
    h = ctypes.c_void_p()
    assert d.lib.gbpa_operator_create(d.ctx, ctypes.byref(desc), ctypes.byref(h)) == -9


def test_indefinite_operator_stops():
    """CGSolver's exit on a non-positive (B r, r): a negative Jacobi inverse
    makes (B r0, r0) < 0; the solve stops at iteration 0, not converged
    (linalg/solvers.cpp:889-906)."""
    from mfem_gb300 import _lib
    from mfem_gb300.pa import PAOperator
    from tests.gpu_util import dev, p
    d = dev()
    fes, integ, _ = setup(3, 2, None)
    A = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata)
    dinv = -torch.ones(fes.ndofs, dtype=torch.float64, device="cuda")
    b = torch.ones_like(dinv)
    x = torch.zeros_like(b)
    info = _lib.SolveInfo()
    st = d.lib.gbpa_pcg_solve(A.handle, p(dinv), p(b), p(x), 1e-10, 0.0, 100, 0, ctypes.byref(info))
    assert st == 0 and info.converged == 0 and info.iterations == 0


@pytest.mark.parametrize("n", [1, 255, 256 * 8 * 152 + 17, 29_503_629])
def test_vec_dot_values_and_reproducibility(n):
    """Vector::operator* (linalg/vector.cpp:1079-1106, reduce in
    general/reducers.hpp:531-594) through gbpa_vec_dot: within a worst-case
    rounding bound of math.fsum of the products (the correctly rounded sum),
    and bit-identical across repeated calls (fixed summation order)."""
    from tests.gpu_util import dev
    d = dev()
    rng = np.random.default_rng(n)
    xh = rng.uniform(-1, 1, n)
    yh = rng.uniform(-1, 1, n)
    x, y = torch.from_numpy(xh).cuda(), torch.from_numpy(yh).cuda()
    r = ctypes.c_double(0.0)
    assert d.lib.gbpa_vec_dot(d.ctx, n, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                              ctypes.byref(r)) == 0
    exact = math.fsum((xh * yh).tolist())
    # worst case: each thread's grid-stride chain (at most n / 1e4 terms for
    # the >= 1e4 threads the kernel runs at these sizes), then two tree levels
    # of depth <= 32 each, every step rounding once (2^-53 relative) with
    # partial sums bounded by sum |x_i y_i|
    k = n / 1e4 + 64
    bound = k * 2.0 ** -53 * float(np.sum(np.abs(xh * yh)))
    assert abs(r.value - exact) <= bound
    vals = set()
    for _ in range(3):
        r2 = ctypes.c_double(0.0)
        assert d.lib.gbpa_vec_dot(d.ctx, n, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                  ctypes.byref(r2)) == 0
        vals.add(r2.value)
    assert vals == {r.value}


@pytest.mark.parametrize("n", [1, 255, 256 * 8 * 152 + 17, 29_503_629])
def test_vec_add_values(n):
    """add(x, a, y, z): z = x + a*y (linalg/vector.cpp:414-600) through
    gbpa_vec_add, against numpy in float64: equal up to the one rounding a
    fused multiply-add saves (at most one ulp of |x| + |a y|); z may alias x."""
    from tests.gpu_util import dev
    d = dev()
    rng = np.random.default_rng(n + 1)
    xh = rng.uniform(-1, 1, n)
    yh = rng.uniform(-1, 1, n)
    a = -0.7310581
    x, y = torch.from_numpy(xh).cuda(), torch.from_numpy(yh).cuda()
    z = torch.full_like(x, float("nan"))
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    assert d.lib.gbpa_vec_add(d.ctx, n, P(x), a, P(y), P(z)) == 0
    torch.cuda.synchronize()
    ref = xh + a * yh
    tol = 2.0 ** -52 * (np.abs(xh) + np.abs(a * yh))
    assert np.all(np.abs(z.cpu().numpy() - ref) <= tol)
    # in place: x = x + a*y
    assert d.lib.gbpa_vec_add(d.ctx, n, P(x), a, P(y), P(x)) == 0
    torch.cuda.synchronize()
    assert np.array_equal(x.cpu().numpy(), z.cpu().numpy())
