"""The oracle's p-multigrid restatement (p-transfer, Chebyshev smoother,
V-cycle, MG-preconditioned CG) pinned against the reference's own outputs on
the pmg4_p124 fixture (orders 1, 2, 4 on a jittered 4^3 mesh, lognormal
kappa; made by tests/golden/make_golden.py through MFEM's
TensorProductPRefinementTransferOperator, OperatorChebyshevSmoother,
Multigrid and CGSolver)."""
import numpy as np
import numpy.polynomial.chebyshev as C
import pytest

from tests import oracle_lib
from tests.conftest import load_golden

ORDERS = (1, 2, 4)


def levels_from_golden(g, lambdas=None):
    lam = g["lambda"] if lambdas is None else lambdas
    out = []
    ne = int(g["meta"][0])
    for l, p in enumerate(ORDERS):
        k = f"l{l}_"
        ndofs = g[k + "offsets"].size - 1
        out.append(oracle_lib.mg_level(ne, ndofs, p + 1, p + 2, g[k + "gather_map"], g[k + "offsets"],
                                       g[k + "indices"], g[k + "B"], g[k + "G"], g[k + "qdata"], g[k + "ess"],
                                       diag=g.get(k + "diag"), lam=float(lam[l - 1]) if l else 0.0,
                                       Bi=g.get(k + "Bi")))
    return out


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def g():
    return load_golden("pmg4_p124")


def test_transfer_tables_are_coarse_basis_at_fine_nodes(oracle, g):
    """The transfer table is the coarse Lagrange basis (Gauss-Lobatto nodes)
    at the fine element's lexicographic Gauss-Lobatto nodes."""
    for l in (1, 2):
        dc, df = ORDERS[l - 1] + 1, ORDERS[l] + 1
        B, _ = oracle.basis_tables(oracle.gauss_lobatto(dc), oracle.gauss_lobatto(df))
        assert np.abs(B.ravel(order="F") - g[f"l{l}_Bi"]).max() < 1e-14


def test_prolongation_and_restriction(oracle, g):
    lv = levels_from_golden(g)
    for l in (1, 2):
        k = f"l{l}_"
        assert rel(oracle.ptransfer_mult(lv[l - 1], lv[l], g[k + "P_x"]), g[k + "P_y"]) < 1e-14
        assert rel(oracle.ptransfer_mult_transpose(lv[l - 1], lv[l], g[k + "Pt_x"]), g[k + "Pt_y"]) < 1e-14


def test_boolean_mask_counts_each_dof_once(oracle, g):
    off, ind = g["l2_offsets"], g["l2_indices"]
    import ctypes
    m = np.zeros(ind.size)
    oracle.lib.or_boolean_mask(off.size - 1, ind.size, oracle_lib._ptr(off), oracle_lib._ptr(ind),
                               oracle_lib._ptr(m))
    assert m.sum() == off.size - 1
    assert all(m[ind[off[i]]] == 1.0 for i in range(0, off.size - 1, 97))


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_chebyshev_polynomial(oracle, order):
    """1 - t p(t) is the scaled Chebyshev polynomial T_k((theta - t)/delta) /
    T_k(theta/delta) on [0.3, 1.2] lambda (the reference's closed forms for
    orders 1-5 are this polynomial's coefficients)."""
    lam = 2.7
    c = oracle.chebyshev_coeffs(order, lam)
    up, lo = 1.2 * lam, 0.3 * lam
    th, de = 0.5 * (up + lo), 0.5 * (up - lo)
    t = np.linspace(0.0, 1.3 * lam, 37)
    p = np.polynomial.polynomial.polyval(t, c)
    Tk = C.Chebyshev.basis(order)
    assert np.abs((1.0 - t * p) - Tk((th - t) / de) / Tk(th / de)).max() < 1e-12


def test_chebyshev_smoother(oracle, g):
    lv = levels_from_golden(g)
    for l in (1, 2):
        k = f"l{l}_"
        assert rel(oracle.chebyshev_mult(lv[l], 2, g[k + "cheb_x"]), g[k + "cheb_y"]) < 1e-13


def test_power_method_close_to_reference(oracle, g):
    """The estimate from a different (splitmix64) start vector after the same
    10 steps is within a few percent of the reference's (its start vector
    comes from the C library's rand())."""
    lv = levels_from_golden(g)
    for l in (1, 2):
        lam = oracle.power_method(lv[l], 10, 1e-8, 12345)
        assert abs(lam - g["lambda"][l - 1]) < 0.05 * g["lambda"][l - 1]


def test_vcycle(oracle, g):
    lv = levels_from_golden(g)
    assert rel(oracle.mg_mult(lv, g["B_rhs"]), g["mg_b"]) < 1e-12


def test_mg_pcg(oracle, g):
    lv = levels_from_golden(g)
    x, it, fn, conv = oracle.mg_pcg(lv, g["B_rhs"], rel_tol=1e-10, max_it=200)
    assert conv
    assert abs(it - int(g["cg_info"][0])) <= 1
    assert rel(x, g["X"]) < 1e-10
