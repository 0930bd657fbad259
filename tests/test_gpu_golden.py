"""GPU parity against the reference's own outputs (golden fixtures generated by
MFEM's CPU partial-assembly path) and against the CPU oracle. Every call goes
through the C ABI of libgbpa.so. Tolerances: integer maps and gathers are
bit-exact; FP64 operators 1e-12 relative L2 (the reference's MFEM_Approx bar);
FP32 applies 1e-5."""
import numpy as np
import pytest
import torch

from tests.conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu

CASES = [c for c in golden_cases() if c != "cfg1_solve"]


def meta(g):
    ne, ndofs, D, Q, cdim, _, n = (int(v) for v in g["meta"])
    return ne, ndofs, D, Q, cdim


@pytest.mark.parametrize("case", golden_cases())
def test_restriction_build_and_gather_scatter(case):
    from tests.gpu_util import T, H, p, call, zeros
    g = load_golden(case)
    ne, ndofs, D, Q, _ = meta(g)
    nd = D ** 3
    off = torch.empty(ndofs + 1, dtype=torch.int32, device="cuda")
    ind = torch.empty(ne * nd, dtype=torch.int32, device="cuda")
    gm = torch.empty(ne * nd, dtype=torch.int32, device="cuda")
    call("gbpa_restriction_build_device", ne, nd, ndofs, p(T(g["elem_dofs"])), p(T(g["dof_map"])),
         p(off), p(ind), p(gm))
    assert np.array_equal(H(gm), g["gather_map"])
    assert np.array_equal(H(off), g["offsets"])
    assert np.array_equal(H(ind), g["indices"])
    x = T(g["x"])
    xE = zeros(ne * nd)
    call("gbpa_restriction_mult", ne, nd, 1, 0, ndofs, p(gm), p(x), p(xE))
    if "xE" in g:
        assert np.array_equal(H(xE), g["xE"])
    # transpose: sums in CSR order exactly like the reference -> bit-exact vs oracle
    from tests import oracle_lib
    o = oracle_lib.load()
    y = zeros(ndofs)
    call("gbpa_restriction_mult_transpose", ne, nd, 1, 0, ndofs, p(off), p(ind), p(xE), p(y), 0)
    yo = o.restriction_mult_transpose(nd, ndofs, g["offsets"], g["indices"], H(xE))
    assert np.array_equal(H(y), yo)
    ya = zeros(ndofs)
    call("gbpa_restriction_abs_mult_transpose", ne, nd, 1, 0, ndofs, p(off), p(ind), p(xE), p(ya))
    assert np.array_equal(H(ya), o.restriction_abs_mult_transpose(nd, ndofs, g["offsets"], g["indices"], H(xE)))


@pytest.mark.parametrize("case", golden_cases())
def test_geometric_factors(case):
    from tests.gpu_util import T, H, p, call, zeros, relerr
    g = load_golden(case)
    ne, ndofs, D, Q, _ = meta(g)
    dg = int(round((g["nodesE"].size / (3 * ne)) ** (1 / 3)))
    J = zeros(Q ** 3 * 9 * ne)
    call("gbpa_geom_jacobians3d", ne, dg, Q, p(T(g["Bg"])), p(T(g["Gg"])), p(T(g["nodesE"])), p(J))
    if "J" in g:
        assert relerr(H(J), g["J"]) < 1e-14
    det = zeros(Q ** 3 * ne)
    call("gbpa_geom_determinants3d", ne, dg, Q, p(T(g["Bg"])), p(T(g["Gg"])), p(T(g["nodesE"])), p(det))
    assert relerr(H(det), g["detJ"]) < 1e-14


@pytest.mark.parametrize("case", CASES)
def test_diffusion_setup_apply_diagonal(case):
    from tests.gpu_util import T, H, p, call, zeros, relerr
    g = load_golden(case)
    ne, ndofs, D, Q, cdim = meta(g)
    symm = 0 if cdim == 9 else 1
    S = 6 if symm else 9
    qd = zeros(Q ** 3 * S * ne)
    C = T(g["coeff"])
    call("gbpa_diffusion_setup3d", ne, Q, cdim, p(T(g["W"])), p(T(g["J"])), p(C), C.numel(), p(qd))
    assert relerr(H(qd), g["qdata_diff"]) < 1e-14
    # fused nodes -> qdata (J never stored)
    dg = int(round((g["nodesE"].size / (3 * ne)) ** (1 / 3)))
    qd2 = zeros(Q ** 3 * S * ne)
    call("gbpa_diffusion_setup3d_nodes", ne, dg, Q, cdim, p(T(g["W"])), p(T(g["Bg"])), p(T(g["Gg"])),
         p(T(g["nodesE"])), p(C), C.numel(), p(qd2))
    assert relerr(H(qd2), g["qdata_diff"]) < 1e-13
    B, G = T(g["B"]), T(g["G"])
    qref = T(g["qdata_diff"])
    yE = zeros(ne * D ** 3)
    call("gbpa_diffusion_apply3d", ne, symm, D, Q, p(B), p(G), None, None, p(qref), p(T(g["xE"])), p(yE))
    assert relerr(H(yE), g["yE_diff"]) < 1e-12
    # accumulate semantics: a second call adds
    call("gbpa_diffusion_apply3d", ne, symm, D, Q, p(B), p(G), None, None, p(qref), p(T(g["xE"])), p(yE))
    assert relerr(H(yE), 2 * g["yE_diff"]) < 1e-12
    dE = zeros(ne * D ** 3)
    call("gbpa_diffusion_diagonal3d", ne, symm, D, Q, p(B), p(G), p(qref), p(dE))
    assert relerr(H(dE), g["diagE_diff"]) < 1e-12
    # FP32 apply
    y32 = zeros(ne * D ** 3, torch.float32)
    call("gbpa_diffusion_apply3d_f32", ne, symm, D, Q, p(B.float()), p(G.float()), p(qref.float()),
         p(T(g["xE"]).float()), p(y32))
    assert relerr(H(y32), g["yE_diff"]) < 1e-5


@pytest.mark.parametrize("case", CASES)
def test_diffusion_operator_lvector(case):
    """PABilinearFormExtension::Mult (L->L) and AssembleDiagonal through the
    fused operator, against BilinearForm::Mult / AssembleDiagonal outputs."""
    from mfem_gb300.pa import ElementRestriction, PAOperator
    from tests.gpu_util import T, H, zeros, relerr, dev
    dev()
    g = load_golden(case)
    ne, ndofs, D, Q, cdim = meta(g)
    R = ElementRestriction.from_maps(ne, D ** 3, ndofs, g["gather_map"], g["offsets"], g["indices"])
    op = PAOperator(0, R, D, Q, T(g["B"]), T(g["G"]), T(g["qdata_diff"]), symm=(cdim != 9))
    y = zeros(ndofs)
    op.Mult(T(g["x"]), y)
    assert relerr(H(y), g["y_diff"]) < 1e-12
    d = zeros(ndofs)
    op.AssembleDiagonal(d)
    assert relerr(H(d), g["diag_diff"]) < 1e-12
    op32 = PAOperator(0, R, D, Q, T(g["B"]), T(g["G"]), T(g["qdata_diff"]), symm=(cdim != 9), precision=1)
    y32 = zeros(ndofs, torch.float32)
    op32.Mult(T(g["x"]).float(), y32)
    assert relerr(H(y32), g["y_diff"]) < 1e-5


@pytest.mark.parametrize("case", CASES)
def test_mass_setup_apply_diagonal(case):
    from mfem_gb300.pa import ElementRestriction, PAOperator
    from tests.gpu_util import T, H, p, call, zeros, relerr
    g = load_golden(case)
    ne, ndofs, D, Q, _ = meta(g)
    qm = zeros(Q ** 3 * ne)
    C = T(g["coeff_mass"])
    call("gbpa_mass_setup3d", ne, Q ** 3, p(T(g["W"])), p(T(g["detJ"])), p(C), C.numel(), 1, p(qm))
    assert relerr(H(qm), g["qdata_mass"]) < 1e-14
    B = T(g["B"])
    yE = zeros(ne * D ** 3)
    call("gbpa_mass_apply3d", ne, D, Q, p(B), None, p(qm), p(T(g["xE"])), p(yE))
    assert relerr(H(yE), g["yE_mass"]) < 1e-12
    R = ElementRestriction.from_maps(ne, D ** 3, ndofs, g["gather_map"], g["offsets"], g["indices"])
    op = PAOperator(1, R, D, Q, B, T(g["G"]), qm)
    y = zeros(ndofs)
    op.Mult(T(g["x"]), y)
    assert relerr(H(y), g["y_mass"]) < 1e-12
    d = zeros(ndofs)
    op.AssembleDiagonal(d)
    assert relerr(H(d), g["diag_mass"]) < 1e-12
    y32 = zeros(ne * D ** 3, torch.float32)
    call("gbpa_mass_apply3d_f32", ne, D, Q, p(B.float()), p(qm.float()), p(T(g["xE"]).float()), p(y32))
    assert relerr(H(y32), g["yE_mass"]) < 1e-5


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", ["diffusion", "mass"])
def test_double_float_operator(case, kind):
    """GBPA_F64X2: FP64 data applied with double-float arithmetic on the FP32
    pipes must meet the FP64 parity bar (1e-12 relative L2) against the
    reference's BilinearForm::Mult."""
    from mfem_gb300.pa import ElementRestriction, PAOperator
    from tests.gpu_util import T, H, zeros, relerr, dev
    dev()
    g = load_golden(case)
    ne, ndofs, D, Q, cdim = meta(g)
    if D > 10 or Q > 10:
        pytest.skip("double-float kernels cover D1D, Q1D <= 10")
    R = ElementRestriction.from_maps(ne, D ** 3, ndofs, g["gather_map"], g["offsets"], g["indices"])
    if kind == "diffusion":
        op = PAOperator(0, R, D, Q, T(g["B"]), T(g["G"]), T(g["qdata_diff"]), symm=(cdim != 9), precision=2)
        ref = g["y_diff"]
    else:
        op = PAOperator(1, R, D, Q, T(g["B"]), T(g["G"]), T(g["qdata_mass"]), precision=2)
        ref = g["y_mass"]
    y = zeros(ndofs)
    op.Mult(T(g["x"]), y)
    assert relerr(H(y), ref) < 1e-12
