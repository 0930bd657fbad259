"""VectorDiffusionIntegrator PA (vdim 3, scalar and vector coefficients) on
the GPU against the reference's own vector apply on the golden cases: the
setup from the fixture's Jacobians and coefficient, the E-vector apply, and
the L-vector product through the vdim-3 restriction (byNODES)."""
import numpy as np
import pytest

from tests.conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu

CASES = [c for c in golden_cases() if c.endswith("_fn") or c.endswith("_vec")]


@pytest.mark.parametrize("case", CASES)
def test_vector_diffusion_matches_reference(case):
    from tests.gpu_util import T, H, p, call, zeros, relerr
    g = load_golden(case)
    ne, ndofs, D, Q, cdim = (int(v) for v in g["meta"][:5])
    Q3, D3 = Q ** 3, D ** 3
    qd = zeros(Q3 * 6 * 3 * ne)
    C = T(g["coeff"])
    call("gbpa_vector_diffusion_setup3d", ne, Q, 3, cdim, p(T(g["W"])), p(T(g["J"])), p(C), C.numel(), p(qd))
    yE = zeros(ne * 3 * D3)
    call("gbpa_vector_diffusion_apply3d", ne, 3, D, Q, p(T(g["B"])), p(T(g["G"])), p(qd), p(T(g["vec_xE"])), p(yE))
    assert relerr(H(yE), g["vec_yE"]) < 1e-12
    # L -> L through the vdim-3 restriction (byNODES) of the same maps
    gm, off, ind = T(g["gather_map"]), T(g["offsets"]), T(g["indices"])
    xE = zeros(ne * 3 * D3)
    call("gbpa_restriction_mult", ne, D3, 3, 0, ndofs, p(gm), p(T(g["vec_x"])), p(xE))
    assert relerr(H(xE), g["vec_xE"]) == 0.0
    yE.zero_()
    call("gbpa_vector_diffusion_apply3d", ne, 3, D, Q, p(T(g["B"])), p(T(g["G"])), p(qd), p(xE), p(yE))
    y = zeros(3 * ndofs)
    call("gbpa_restriction_mult_transpose", ne, D3, 3, 0, ndofs, p(off), p(ind), p(yE), p(y), 0)
    assert relerr(H(y), g["vec_y"]) < 1e-12


@pytest.mark.parametrize("case", CASES)
def test_vector_mass_matches_reference(case):
    from tests.gpu_util import T, H, p, call, zeros, relerr
    g = load_golden(case)
    ne, ndofs, D, Q, cdim = (int(v) for v in g["meta"][:5])
    Q3, D3 = Q ** 3, D ** 3
    qd = zeros(Q3 * cdim * ne)
    C = T(g["vmass_coeff"])
    call("gbpa_vector_mass_setup3d", ne, Q, 3, cdim, p(T(g["W"])), p(T(g["J"])), p(C), C.numel(), p(qd))
    yE = zeros(ne * 3 * D3)
    call("gbpa_vector_mass_apply3d", ne, 3, cdim, D, Q, p(T(g["B"])), p(qd), p(T(g["vec_xE"])), p(yE))
    assert relerr(H(yE), g["vmass_yE"]) < 1e-12
    y = zeros(3 * ndofs)
    call("gbpa_restriction_mult_transpose", ne, D3, 3, 0, ndofs, p(T(g["offsets"])), p(T(g["indices"])), p(yE),
         p(y), 0)
    assert relerr(H(y), g["vmass_y"]) < 1e-12


def test_vector_matrix_coefficient_matches_reference():
    """Matrix coefficient (components coupled): VectorDiffusionIntegrator and
    VectorMassIntegrator PA through gbpa_vector_diffusion_setup3d /
    gbpa_vector_diffusion_apply3d_coeff and gbpa_vector_mass_setup3d /
    gbpa_vector_mass_apply3d with coeff_vdim 9, against the reference's own
    vector applies (E-vector and L-vector through the vdim-3 restriction)."""
    from tests.gpu_util import T, H, p, call, zeros, relerr
    g = load_golden("jit2_p2_nonsym")
    ne, ndofs, D, Q = (int(v) for v in g["meta"][:4])
    Q3, D3 = Q ** 3, D ** 3
    C = T(g["vmat_coeff"])
    qd = zeros(Q3 * 6 * 9 * ne)
    call("gbpa_vector_diffusion_setup3d", ne, Q, 3, 9, p(T(g["W"])), p(T(g["J"])), p(C), C.numel(), p(qd))
    xE = T(g["vec_xE"])
    yE = zeros(ne * 3 * D3)
    call("gbpa_vector_diffusion_apply3d_coeff", ne, 3, 9, D, Q, p(T(g["B"])), p(T(g["G"])), p(qd), p(xE), p(yE))
    assert relerr(H(yE), g["vmat_yE"]) < 1e-12
    y = zeros(3 * ndofs)
    call("gbpa_restriction_mult_transpose", ne, D3, 3, 0, ndofs, p(T(g["offsets"])), p(T(g["indices"])), p(yE),
         p(y), 0)
    assert relerr(H(y), g["vmat_y"]) < 1e-12
    # vector mass, same coefficient
    qm = zeros(Q3 * 9 * ne)
    call("gbpa_vector_mass_setup3d", ne, Q, 3, 9, p(T(g["W"])), p(T(g["J"])), p(C), C.numel(), p(qm))
    yE.zero_()
    call("gbpa_vector_mass_apply3d", ne, 3, 9, D, Q, p(T(g["B"])), p(qm), p(xE), p(yE))
    assert relerr(H(yE), g["vmatmass_yE"]) < 1e-12
    call("gbpa_restriction_mult_transpose", ne, D3, 3, 0, ndofs, p(T(g["offsets"])), p(T(g["indices"])), p(yE),
         p(y), 0)
    assert relerr(H(y), g["vmatmass_y"]) < 1e-12
    # the scalar/vector paths of the _coeff entry point are the plain vector apply
    from tests.gpu_util import dev
    d = dev()
    assert d.lib.gbpa_vector_diffusion_apply3d_coeff(d.ctx, ne, 3, 4, D, Q, None, None, None, None, None) == -1
