"""Domain-integrator element markers (PABilinearFormExtension::
AddMultWithMarkers, fem/bilinearform_ext.cpp:530-550,753-774,807-847) through
gbpa_operator_set_element_markers: only elements whose attribute is marked
contribute to Mult and to AssembleDiagonal. Checked against the reference's
own marked Mult and diagonal (golden fixture), and against the oracle's
restatement for more marker sets, for the native FP64 and double-float
operators, constrained and not, CSR and atomic scatter; removing the markers
restores the full operator; an attribute beyond the marker array is an index
error."""
import numpy as np
import pytest
import torch

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def _setup(case="jit3_p3_fn"):
    from mfem_gb300.pa import ElementRestriction
    from tests.gpu_util import T
    g = load_golden(case)
    ne, ndofs, D, Q = (int(v) for v in g["meta"][:4])
    R = ElementRestriction.from_maps(ne, D ** 3, ndofs, g["gather_map"], g["offsets"], g["indices"])
    return g, ne, ndofs, D, Q, R, T(g["B"]), T(g["G"]), T(g["qdata_diff"])


@pytest.mark.parametrize("precision", [0, 2])
@pytest.mark.parametrize("scatter", [0, 1])
def test_markers_mult_matches_oracle(oracle, precision, scatter):
    from mfem_gb300.pa import PAOperator
    from tests.gpu_util import T, H
    g, ne, ndofs, D, Q, R, B, G, qd = _setup()
    op = PAOperator(0, R, D, Q, B, G, qd, precision=precision, scatter=scatter)
    rng = np.random.default_rng(11)
    attr = rng.integers(1, 4, ne).astype(np.int32)
    x = T(g["x"])
    y = torch.empty_like(x)
    args = (0, ne, ndofs, True, D, Q, g["gather_map"], g["offsets"], g["indices"], g["B"], g["G"], g["qdata_diff"])
    for markers in ([1, 0, 1], [0, 1, 0], [0, 0, 0], [1, 1, 1]):
        op.SetElementMarkers(attr, markers)
        op.Mult(x, y)
        ref = oracle.pa_mult_markers(*args, attr, markers, g["x"])
        if not any(markers):
            assert np.abs(H(y)).max() == 0.0
        else:
            assert np.linalg.norm(H(y) - ref) / np.linalg.norm(ref) < 1e-12
    op.SetElementMarkers(None, None)
    op.Mult(x, y)
    assert np.linalg.norm(H(y) - g["y_diff"]) / np.linalg.norm(g["y_diff"]) < 1e-12


@pytest.mark.parametrize("precision", [0, 2])
def test_markers_against_reference_fixture(precision):
    """Mult and AssembleDiagonal of the marked operator against the
    reference's own output for AddDomainIntegrator(integ, marker) (element
    attributes 1 + e % 3, marker {1, 0, 1})."""
    from mfem_gb300.pa import PAOperator
    from tests.gpu_util import T, H
    g, ne, ndofs, D, Q, R, B, G, qd = _setup()
    op = PAOperator(0, R, D, Q, B, G, qd, precision=precision)
    op.SetElementMarkers(g["elem_attr"].astype(np.int32), g["markers"].astype(np.int32))
    x = T(g["x"])
    y = torch.empty_like(x)
    op.Mult(x, y)
    ref = g["y_diff_markers"]
    assert np.linalg.norm(H(y) - ref) / np.linalg.norm(ref) < 1e-12
    diag = torch.empty(ndofs, dtype=torch.float64, device="cuda")
    op.AssembleDiagonal(diag)
    dref = g["diag_diff_markers"]
    assert np.linalg.norm(H(diag) - dref) / np.linalg.norm(dref) < 1e-12


def test_markers_diagonal_and_constrained(oracle):
    """Marked diagonal = the diagonal of the marked operator (every unit
    vector), and the constrained marked operator keeps y[ess] = x[ess]."""
    from mfem_gb300.pa import PAOperator
    from tests.gpu_util import T, H
    g, ne, ndofs, D, Q, R, B, G, qd = _setup("cart2_p2_one")
    attr = (np.arange(ne) % 2 + 1).astype(np.int32)
    markers = [0, 1]
    op = PAOperator(0, R, D, Q, B, G, qd)
    op.SetElementMarkers(attr, markers)
    diag = torch.empty(ndofs, dtype=torch.float64, device="cuda")
    op.AssembleDiagonal(diag)
    args = (0, ne, ndofs, True, D, Q, g["gather_map"], g["offsets"], g["indices"], g["B"], g["G"], g["qdata_diff"])
    ref = np.array([oracle.pa_mult_markers(*args, attr, markers, np.eye(ndofs)[i])[i] for i in range(ndofs)])
    assert np.linalg.norm(H(diag) - ref) / np.linalg.norm(ref) < 1e-13
    ess = np.array([0, 3, 7], np.int32)
    opc = PAOperator(0, R, D, Q, B, G, qd, ess=ess)
    opc.SetElementMarkers(attr, markers)
    rng = np.random.default_rng(5)
    xh = rng.uniform(-1, 1, ndofs)
    x, y = T(xh), torch.empty(ndofs, dtype=torch.float64, device="cuda")
    opc.Mult(x, y)
    z = xh.copy(); z[ess] = 0.0
    ref = oracle.pa_mult_markers(*args, attr, markers, z)
    ref[ess] = xh[ess]
    assert np.linalg.norm(H(y) - ref) / np.linalg.norm(ref) < 1e-12


def test_markers_reject_attribute_out_of_range():
    from mfem_gb300 import _lib
    from mfem_gb300.pa import PAOperator
    from tests.gpu_util import T, H
    g, ne, ndofs, D, Q, R, B, G, qd = _setup()
    op = PAOperator(0, R, D, Q, B, G, qd)
    attr = np.full(ne, 4, np.int32)
    with pytest.raises(_lib.GbpaError) as e:
        op.SetElementMarkers(attr, [1, 1, 1])
    assert e.value.status == -9
    # the failed call left every element active
    x = T(g["x"]); y = torch.empty_like(x)
    op.Mult(x, y)
    assert np.linalg.norm(H(y) - g["y_diff"]) / np.linalg.norm(g["y_diff"]) < 1e-12
