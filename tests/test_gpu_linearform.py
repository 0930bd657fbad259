"""Device LinearForm assembly (gbpa_domain_lf3d, DomainLFIntegrator through
LinearFormExtension) against the reference's own device-path assembly of
DomainLFIntegrator(kappa) on the golden cases: from the fixture's inputs
through the C ABI, and end to end through the package's LinearForm on the
same meshes."""
import numpy as np
import pytest
import torch

from tests.conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu

CASES = [c for c in golden_cases() if c != "cfg1_solve"]
# (n, p, jitter, curved) of the golden meshes made by the golden driver
MESHES = {"cart2_p2_one": (2, 2, 0.0, False), "cart2_p1_const": (2, 1, 0.0, False),
          "jit3_p3_fn": (3, 3, 0.1, False), "jit2_p4_vec": (2, 4, 0.1, False), "jit2_p4_sym": (2, 4, 0.1, False),
          "jit2_p2_nonsym": (2, 2, 0.1, False), "jit2_p6_fn": (2, 6, 0.1, False), "cart1_p8_one": (1, 8, 0.0, False),
          "jit1_p7_fn": (1, 7, 0.1, False), "curv2_p3_fn": (2, 3, 0.0, True),
          "jit2_p5_fn": (2, 5, 0.1, False), "curv2_p5_fn": (2, 5, 0.0, True)}


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("case", CASES)
def test_domain_lf_from_reference_inputs(case):
    from tests.gpu_util import T, H, p, call, zeros
    g = load_golden(case)
    ne, ndofs, D = int(g["meta"][0]), int(g["meta"][1]), int(g["meta"][2])
    b = zeros(ndofs)
    call("gbpa_domain_lf3d", ne, D, D, p(T(g["lf_B"])), p(T(g["lf_W"])), p(T(g["lf_detJ"])), p(T(g["lf_coeff"])),
         g["lf_coeff"].size, ndofs, p(T(g["offsets"])), p(T(g["indices"])), p(b))
    assert rel(H(b), g["lf_fn"]) < 1e-13


def reference_dof_of(g, n, nd, our_gather_map):
    """For each of the package's dofs, the reference dof at the same place.
    The reference's MakeCartesian3D numbers vertices lexicographically (as the
    package does) but orders elements along a space-filling curve, and numbers
    dofs by vertices, edges, faces and interiors; both gather maps list an
    element's dofs in the same lexicographic order. So element e of the
    reference is the package's element at the lattice position of its first
    corner vertex, and slot l of the two elements holds the same dof."""
    ev = np.asarray(g["elem_vertices"]).reshape(-1, 8)
    v0 = ev[:, 0]
    i, j, k = v0 % (n + 1), (v0 // (n + 1)) % (n + 1), v0 // (n + 1) ** 2
    ours = i + n * (j + n * k)                      # package element of each reference element
    ref_gm = np.asarray(g["gather_map"]).reshape(-1, nd)
    our_gm = np.asarray(our_gather_map).reshape(-1, nd)[ours]
    assert (ref_gm >= 0).all() and (our_gm >= 0).all()
    perm = np.full(our_gm.max() + 1, -1, np.int64)
    perm[our_gm.reshape(-1)] = ref_gm.reshape(-1)
    # a consistent bijection: every package dof gets exactly one reference dof
    assert (perm >= 0).all()
    pairs = np.unique(np.stack([our_gm.reshape(-1), ref_gm.reshape(-1)]), axis=1)
    assert pairs.shape[1] == perm.size and np.unique(perm).size == perm.size
    return perm


@pytest.mark.parametrize("case", ["jit3_p3_fn", "jit2_p6_fn", "curv2_p3_fn", "cart1_p8_one", "curv2_p5_fn"])
def test_linear_form_end_to_end(case):
    """Geometry, kappa at the rule's points and the assembly all on the
    device from the package's own mesh, compared entry by entry with the
    reference's vector through the dof correspondence (reference_dof_of)."""
    from mfem_gb300 import fem
    from mfem_gb300.pa import DomainLFIntegrator, FiniteElementSpace, LinearForm
    from tests.gpu_util import dev
    dev()
    g = load_golden(case)
    n, pdeg, jit, curved = MESHES[case]
    mesh = fem.CartesianMesh(n, jitter=jit, seed=1, curved=curved)
    fes = FiniteElementSpace(mesh, pdeg)
    lf = LinearForm(fes)
    lf.AddDomainIntegrator(DomainLFIntegrator("kappa"))
    b = lf.Assemble(modes=fem.kappa_modes(3))
    perm = reference_dof_of(g, n, (pdeg + 1) ** 3, fes.GetElementRestriction().gather_map.cpu().numpy())
    assert rel(b.cpu().numpy(), np.asarray(g["lf_fn"])[perm]) < 1e-13


def test_linear_form_of_one_integrates_the_volume():
    """With f = 1 the entries sum to |Omega| = 1 (the basis is a partition of
    unity), on a jittered 10^3 mesh at p = 4."""
    from mfem_gb300 import fem
    from mfem_gb300.pa import DomainLFIntegrator, FiniteElementSpace, LinearForm
    from tests.gpu_util import dev
    dev()
    fes = FiniteElementSpace(fem.CartesianMesh(10, jitter=0.1, seed=3), 4)
    lf = LinearForm(fes)
    lf.AddDomainIntegrator(DomainLFIntegrator(None))
    b = lf.Assemble()
    assert abs(float(b.sum()) - 1.0) < 1e-13


def test_lognormal_coefficient_kernel_matches_numpy():
    """gbpa_coefficient_lognormal3d against the same field evaluated by numpy
    at the same quadrature coordinates (curved order-3 geometry)."""
    import ctypes
    import numpy as np
    import torch
    from mfem_gb300 import fem
    from mfem_gb300.pa import FiniteElementSpace, _geometry
    from tests.gpu_util import dev
    d = dev()
    mesh = fem.CartesianMesh(3, curved=True)
    fes = FiniteElementSpace(mesh, 2)
    t = fem.Tables(2, 5)
    modes = fem.kappa_modes(3)
    geom = _geometry(fes, t, modes)
    ne, nq = fes.ne, 5 ** 3
    XQ = torch.empty(nq * 3 * ne, dtype=torch.float64, device="cuda")
    P = lambda a: ctypes.c_void_p(a.data_ptr())
    assert d.lib.gbpa_geom_coordinates3d(d.ctx, ne, geom["dg"], 5, P(geom["Bg"]), P(geom["X"]), P(XQ)) == 0
    k = np.ascontiguousarray(modes[0], np.int32).reshape(-1)
    phi = np.ascontiguousarray(modes[1], np.float64)
    out = torch.empty(nq * ne, dtype=torch.float64, device="cuda")
    assert d.lib.gbpa_coefficient_lognormal3d(d.ctx, ne, nq, P(XQ), len(phi),
                                              k.ctypes.data_as(ctypes.c_void_p),
                                              phi.ctypes.data_as(ctypes.c_void_p), 0.5, P(out)) == 0
    xyz = XQ.cpu().numpy().reshape(ne, 3, nq).transpose(0, 2, 1)
    ref = fem.kappa_eval(xyz, modes).reshape(-1)
    assert np.max(np.abs(out.cpu().numpy() - ref) / ref) < 1e-13
    # invalid arguments
    assert d.lib.gbpa_coefficient_lognormal3d(d.ctx, ne, nq, P(XQ), 65, k.ctypes.data_as(ctypes.c_void_p),
                                              phi.ctypes.data_as(ctypes.c_void_p), 0.5, P(out)) < 0
