"""The CPU oracle is pinned against golden vectors produced by the reference
itself (tests/golden/*.npz, made by tests/golden/make_golden.py from MFEM's own
partial-assembly path). Tolerances follow the reference's unit tests
(MFEM_Approx 1e-12) except where noted; integer maps are bit-exact."""
import numpy as np
import pytest

from tests.conftest import golden_cases, load_golden

CASES = golden_cases()


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def meta(g):
    ne, ndofs, D, Q, cdim, ckind, n = (int(v) for v in g["meta"])
    return ne, ndofs, D, Q, cdim


def tensor_weights(w):
    Q = len(w)
    return np.einsum("k,j,i->kji", w, w, w).reshape(Q ** 3)


@pytest.mark.parametrize("case", CASES)
def test_restriction_maps_bit_exact(oracle, case):
    g = load_golden(case)
    ne, ndofs, D, Q, _ = meta(g)
    off, ind, gm = oracle.restriction_build(ne, D ** 3, ndofs, g["elem_dofs"], g["dof_map"])
    assert np.array_equal(gm, g["gather_map"])
    assert np.array_equal(off, g["offsets"])
    assert np.array_equal(ind, g["indices"])


@pytest.mark.parametrize("case", CASES)
def test_quadrature_and_basis(oracle, case):
    g = load_golden(case)
    ne, ndofs, D, Q, _ = meta(g)
    xq, wq = oracle.gauss_legendre(Q)
    assert np.allclose(tensor_weights(wq), g["W"], rtol=1e-14, atol=1e-15)
    nodes = oracle.gauss_lobatto(D)
    B, G = oracle.basis_tables(nodes, xq)
    assert np.abs(B - g["B"]).max() < 1e-13
    assert np.abs(G - g["G"]).max() < 1e-12 * max(1.0, np.abs(g["G"]).max())
    # Bt/Gt are the transposes (D, Q)
    assert np.array_equal(g["Bt"].reshape(Q, D, order="C"), g["B"].reshape(D, Q).T)


@pytest.mark.parametrize("case", CASES)
def test_geometric_factors(oracle, case):
    g = load_golden(case)
    ne, ndofs, D, Q, _ = meta(g)
    dg = int(round((g["nodesE"].size / (3 * ne)) ** (1 / 3)))
    J = oracle.geom_jacobians3d(ne, dg, Q, g["Bg"], g["Gg"], g["nodesE"])
    if "J" in g:
        assert relerr(J, g["J"]) < 1e-14
    det = oracle.geom_det3d(ne, J, Q ** 3)
    assert relerr(det, g["detJ"]) < 1e-14


@pytest.mark.parametrize("case", [c for c in CASES if c != "cfg1_solve"])
def test_diffusion_setup_apply_diag(oracle, case):
    g = load_golden(case)
    ne, ndofs, D, Q, cdim = meta(g)
    symm = cdim != 9
    qd = oracle.diffusion_setup3d(ne, Q, cdim, g["W"], g["J"], g["coeff"])
    assert relerr(qd, g["qdata_diff"]) < 1e-14
    yE = oracle.diffusion_apply3d(ne, symm, D, Q, g["B"], g["G"], g["qdata_diff"], g["xE"])
    assert relerr(yE, g["yE_diff"]) < 1e-12
    y = oracle.pa_mult(0, ne, ndofs, symm, D, Q, g["gather_map"], g["offsets"], g["indices"],
                       g["B"], g["G"], g["qdata_diff"], g["x"])
    assert relerr(y, g["y_diff"]) < 1e-12
    dE = oracle.diffusion_diagonal3d(ne, symm, D, Q, g["B"], g["G"], g["qdata_diff"])
    assert relerr(dE, g["diagE_diff"]) < 1e-12
    d = oracle.restriction_abs_mult_transpose(D ** 3, ndofs, g["offsets"], g["indices"], dE)
    assert relerr(d, g["diag_diff"]) < 1e-12


@pytest.mark.parametrize("case", [c for c in CASES if c != "cfg1_solve"])
def test_mass_setup_apply_diag(oracle, case):
    g = load_golden(case)
    ne, ndofs, D, Q, _ = meta(g)
    qm = oracle.mass_setup3d(ne, Q ** 3, g["W"], g["detJ"], g["coeff_mass"])
    assert relerr(qm, g["qdata_mass"]) < 1e-14
    yE = oracle.mass_apply3d(ne, D, Q, g["B"], qm, g["xE"])
    assert relerr(yE, g["yE_mass"]) < 1e-12
    y = oracle.pa_mult(1, ne, ndofs, True, D, Q, g["gather_map"], g["offsets"], g["indices"],
                       g["B"], g["G"], qm, g["x"])
    assert relerr(y, g["y_mass"]) < 1e-12
    dE = oracle.mass_diagonal3d(ne, D, Q, g["B"], qm)
    d = oracle.restriction_abs_mult_transpose(D ** 3, ndofs, g["offsets"], g["indices"], dE)
    assert relerr(d, g["diag_mass"]) < 1e-12


def cfg1_operator(oracle, g):
    ne, ndofs, D, Q, cdim = meta(g)
    dg = int(round((g["nodesE"].size / (3 * ne)) ** (1 / 3)))
    J = oracle.geom_jacobians3d(ne, dg, Q, g["Bg"], g["Gg"], g["nodesE"])
    qd = oracle.diffusion_setup3d(ne, Q, cdim, g["W"], J, g["coeff"])
    return ne, ndofs, D, Q, qd


def test_cfg1_operator_and_jacobi(oracle):
    g = load_golden("cfg1_solve")
    ne, ndofs, D, Q, qd = cfg1_operator(oracle, g)
    y = oracle.pa_mult(0, ne, ndofs, True, D, Q, g["gather_map"], g["offsets"], g["indices"],
                       g["B"], g["G"], qd, g["x"])
    assert relerr(y, g["y_diff"]) < 1e-12
    dE = oracle.diffusion_diagonal3d(ne, True, D, Q, g["B"], g["G"], qd)
    diag = oracle.restriction_abs_mult_transpose(D ** 3, ndofs, g["offsets"], g["indices"], dE)
    assert relerr(diag, g["diag_diff"]) < 1e-12
    ess = g["ess_tdofs"]
    # ConstrainedOperator (DIAG_ONE) applied to x
    z = g["x"].copy(); z[ess] = 0.0
    Ax = oracle.pa_mult(0, ne, ndofs, True, D, Q, g["gather_map"], g["offsets"], g["indices"],
                        g["B"], g["G"], qd, z)
    Ax[ess] = g["x"][ess]
    assert relerr(Ax, g["Ax_constrained"]) < 1e-12
    dinv = 1.0 / diag; dinv[ess] = 1.0
    assert relerr(dinv * g["x"], g["Mx_jacobi"]) < 1e-12


def test_cfg1_pcg_solution(oracle):
    g = load_golden("cfg1_solve")
    ne, ndofs, D, Q, qd = cfg1_operator(oracle, g)
    dE = oracle.diffusion_diagonal3d(ne, True, D, Q, g["B"], g["G"], qd)
    diag = oracle.restriction_abs_mult_transpose(D ** 3, ndofs, g["offsets"], g["indices"], dE)
    ess = g["ess_tdofs"]
    dinv = 1.0 / diag; dinv[ess] = 1.0
    X, it, fn, conv = oracle.pcg_diffusion(ne, ndofs, True, D, Q, g["gather_map"], g["offsets"],
                                           g["indices"], g["B"], g["G"], qd, ess, dinv, g["B_rhs"],
                                           rel_tol=1e-12, max_it=500)
    ref_it, ref_norm, ref_conv = g["cg_info"]
    assert conv and bool(ref_conv)
    assert abs(it - int(ref_it)) <= 1
    assert relerr(X, g["X"]) < 1e-10


@pytest.mark.parametrize("case", [c for c in CASES if c != "cfg1_solve"])
def test_domain_linear_form(oracle, case):
    """DomainLFIntegrator(kappa) assembled through the reference's device
    path (LinearForm::UseFastAssembly) at its default rule (p + 1 Gauss
    points): the oracle's restatement from the rule's inputs, and the basis
    table against the oracle's own."""
    g = load_golden(case)
    ne, ndofs, D, Q, _ = meta(g)
    lq = D     # p + 1 points
    x, _ = oracle.gauss_legendre(lq)
    B, _ = oracle.basis_tables(oracle.gauss_lobatto(D), x)
    assert np.abs(B.ravel(order="F") - g["lf_B"]).max() < 1e-14
    b = oracle.domain_lf3d(ne, D, lq, g["lf_B"], g["lf_W"], g["lf_detJ"], g["lf_coeff"], ndofs,
                           g["offsets"], g["indices"])
    ref = g["lf_fn"]
    assert np.linalg.norm(b - ref) / np.linalg.norm(ref) < 1e-14


@pytest.mark.parametrize("case", [c for c in CASES if c.endswith("_fn") or c.endswith("_vec")])
def test_vector_diffusion_componentwise(oracle, case):
    """VectorDiffusionIntegrator PA (vdim 3) with a scalar or vector
    coefficient is the scalar diffusion operator per component, each with its
    coefficient component: the oracle's scalar setup and apply per component
    reproduce the reference's vector E-vector apply."""
    g = load_golden(case)
    ne, ndofs, D, Q, cdim = meta(g)
    Q3, D3 = Q ** 3, D ** 3
    C = g["coeff"]
    xE = g["vec_xE"].reshape(ne, 3, D3)
    yE = np.zeros_like(xE)
    for i in range(3):
        Ci = C if cdim == 1 else C.reshape(-1, 3)[:, i].copy()
        Di = oracle.diffusion_setup3d(ne, Q, 1, g["W"], g["J"], Ci)
        yE[:, i, :] = oracle.diffusion_apply3d(ne, True, D, Q, g["B"], g["G"], Di,
                                               xE[:, i, :].copy()).reshape(ne, D3)
    ref = g["vec_yE"].reshape(ne, 3, D3)
    assert np.linalg.norm(yE - ref) / np.linalg.norm(ref) < 1e-13


@pytest.mark.parametrize("case", [c for c in CASES if c.endswith("_fn") or c.endswith("_vec")])
def test_vector_mass_componentwise(oracle, case):
    """VectorMassIntegrator PA (vdim 3, scalar or vector coefficient) is the
    scalar mass operator per component with that component's coefficient."""
    g = load_golden(case)
    ne, ndofs, D, Q, cdim = meta(g)
    Q3, D3 = Q ** 3, D ** 3
    C = g["vmass_coeff"]
    xE = g["vec_xE"].reshape(ne, 3, D3)
    yE = np.zeros_like(xE)
    for i in range(3):
        Ci = C if cdim == 1 else C.reshape(-1, 3)[:, i].copy()
        Di = oracle.mass_setup3d(ne, Q3, g["W"], g["detJ"], Ci)
        yE[:, i, :] = oracle.mass_apply3d(ne, D, Q, g["B"], Di, xE[:, i, :].copy()).reshape(ne, D3)
    ref = g["vmass_yE"].reshape(ne, 3, D3)
    assert np.linalg.norm(yE - ref) / np.linalg.norm(ref) < 1e-13


def test_markers_oracle_matches_reference(oracle):
    """The element-marker restatement against the reference's own
    BilinearForm::Mult of a form added with AddDomainIntegrator(integ, marker)
    (element attributes 1 + e % 3, marker {1, 0, 1}; fixture written by
    oracle/ref/golden_driver.cpp)."""
    g = load_golden("jit3_p3_fn")
    ne, ndofs, D, Q = (int(v) for v in g["meta"][:4])
    args = (0, ne, ndofs, True, D, Q, g["gather_map"], g["offsets"], g["indices"], g["B"], g["G"],
            g["qdata_diff"])
    y = oracle.pa_mult_markers(*args, g["elem_attr"], g["markers"], g["x"])
    ref = g["y_diff_markers"]
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-12


def test_markers_oracle_all_and_none_marked(oracle):
    """The element-marker restatement (AddMultWithMarkers) reduces to the
    plain L->L apply when every attribute is marked, gives zero when none
    is, and is additive over a partition of the attributes."""
    g = load_golden("jit3_p3_fn")
    ne, ndofs, D, Q = (int(v) for v in g["meta"][:4])
    args = (0, ne, ndofs, True, D, Q, g["gather_map"], g["offsets"], g["indices"], g["B"], g["G"],
            g["qdata_diff"])
    rng = np.random.default_rng(3)
    attr = rng.integers(1, 4, ne).astype(np.int32)
    full = oracle.pa_mult(*args, g["x"])
    assert np.allclose(oracle.pa_mult_markers(*args, attr, [1, 1, 1], g["x"]), full, rtol=0, atol=1e-13)
    assert np.abs(oracle.pa_mult_markers(*args, attr, [0, 0, 0], g["x"])).max() == 0.0
    part = sum(oracle.pa_mult_markers(*args, attr, m, g["x"]) for m in ([1, 0, 0], [0, 1, 0], [0, 0, 1]))
    assert np.linalg.norm(part - full) / np.linalg.norm(full) < 1e-14
    assert np.allclose(full, g["y_diff"], rtol=0, atol=1e-12 * np.abs(g["y_diff"]).max())


MATRIX_MAP = [0, 3, 6, 1, 4, 7, 2, 5, 8]


def test_vector_matrix_coefficient_componentwise(oracle):
    """VectorDiffusionIntegrator / VectorMassIntegrator PA with a matrix
    coefficient (components coupled through it) is the sum of scalar
    operators, one per coefficient entry: diffusion block b = j + 3 i (source
    i, destination j) with coefficient entry map[b]
    (fem/integ/bilininteg_vecdiffusion_pa.cpp:213-272, .hpp:96-163); mass
    block 3 c + d (source d, destination c) with entry 3 c + d
    (fem/integ/bilininteg_vecmass_pa.cpp:119-160, .hpp:157-170). The scalar
    oracle composed this way reproduces the reference's vector E-vectors."""
    g = load_golden("jit2_p2_nonsym")
    ne, ndofs, D, Q = (int(v) for v in g["meta"][:4])
    Q3, D3 = Q ** 3, D ** 3
    C = np.asarray(g["vmat_coeff"]).reshape(ne * Q3, 9)
    xE = np.asarray(g["vec_xE"]).reshape(ne, 3, D3)
    y = np.zeros((ne, 3, D3))
    ym = np.zeros((ne, 3, D3))
    for i in range(3):
        xi = np.ascontiguousarray(xE[:, i, :]).reshape(-1)
        for j in range(3):
            b = j + 3 * i
            qd = oracle.diffusion_setup3d(ne, Q, 1, g["W"], g["J"], np.ascontiguousarray(C[:, MATRIX_MAP[b]]))
            y[:, j, :] += oracle.diffusion_apply3d(ne, True, D, Q, g["B"], g["G"], qd, xi).reshape(ne, D3)
            bm = 3 * j + i
            qm = oracle.mass_setup3d(ne, Q3, g["W"], g["detJ"], np.ascontiguousarray(C[:, bm]))
            ym[:, j, :] += oracle.mass_apply3d(ne, D, Q, g["B"], qm, xi).reshape(ne, D3)
    ref = np.asarray(g["vmat_yE"])
    assert np.linalg.norm(y.reshape(-1) - ref) / np.linalg.norm(ref) < 1e-13
    refm = np.asarray(g["vmatmass_yE"])
    assert np.linalg.norm(ym.reshape(-1) - refm) / np.linalg.norm(refm) < 1e-13
