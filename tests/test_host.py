"""Host-side discretisation data (mfem_gb300.fem) against the reference's
golden tables and meshes, and the synthetic-input recipe against the one the
golden driver used."""
import numpy as np
import pytest

from mfem_gb300 import fem
from tests.conftest import golden_cases, load_golden


@pytest.mark.parametrize("case", golden_cases())
def test_tables_match_reference(case):
    g = load_golden(case)
    D, Q = int(g["meta"][2]), int(g["meta"][3])
    t = fem.Tables(D - 1, Q)
    assert np.abs(t.B - g["B"]).max() < 1e-13
    assert np.abs(t.G - g["G"]).max() < 1e-12 * max(1, np.abs(g["G"]).max())
    assert np.allclose(t.W, g["W"], rtol=1e-14, atol=1e-16)


@pytest.mark.parametrize("case", golden_cases())
def test_vertices_match_reference(case):
    g = load_golden(case)
    n = int(g["meta"][6])
    jitter = 0.1 if case.startswith("jit") else 0.0
    m = fem.CartesianMesh(n, jitter=jitter, seed=1)
    assert np.array_equal(m.vertices.reshape(-1), g["vertices"])


def test_u01_stream_vectorised_matches_scalar():
    assert np.array_equal(fem.u01_array(7, 50), fem.u01_stream(7, 50))


def test_h1_space_numbering():
    m = fem.CartesianMesh(3)
    s = fem.H1Space(m, 2)
    ed = s.element_dofs().reshape(m.ne, 27)
    assert ed.max() == s.ndofs - 1 and ed.min() == 0
    # every dof appears; interior element dof (1,1,1) belongs to one element
    counts = np.bincount(ed.ravel(), minlength=s.ndofs)
    assert counts.min() >= 1 and counts.max() == 8
    assert len(s.boundary_dofs()) == s.N1 ** 3 - (s.N1 - 2) ** 3


def test_oracle_restriction_on_own_numbering(oracle):
    m = fem.CartesianMesh(4)
    s = fem.H1Space(m, 3)
    off, ind, gm = oracle.restriction_build(m.ne, 64, s.ndofs, s.element_dofs(), None)
    assert np.array_equal(gm, s.element_dofs())
    assert off[-1] == m.ne * 64
