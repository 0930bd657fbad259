"""Host-side checks of the autotuner's table and candidate sets, and of the
bench's algorithmic work accounting (no GPU)."""
import json
import os

import pytest

from tests.conftest import REPO


def tuning():
    with open(os.path.join(REPO, "mfem_gb300", "tuning.json")) as f:
        return json.load(f)


def test_tuning_table_entries_are_launchable():
    """Every 2D-slab entry fits a 1024-thread block with blockDim.z <= 64 and
    the autotuner's shared-memory budget; every 3D-layout entry names a
    diffusion order that has a compile-time 3D kernel and fits the 3D limits."""
    from mfem_gb300 import autotune as at
    t = tuning()
    assert t["nbz"], "empty tuning table"
    for k, nbz in t["nbz"].items():
        kind, prec, D, Q = k.split(":")
        D, Q = int(D), int(Q)
        assert kind in at.KINDS and prec in at.PRECS
        assert 1 <= nbz <= 64 and nbz * Q * Q <= 1024, k
        assert nbz in at.candidates(kind, prec, D, Q), k
    for k, nbz in t.get("layout3d", {}).items():
        kind, prec, D, Q = k.split(":")
        D, Q = int(D), int(Q)
        assert (D, Q) in at.DQ3, k
        assert nbz in at.candidates_3d(prec, D, Q, kind), k
        assert nbz * Q <= 64 and nbz * Q ** 3 <= 1024, k


def test_3d_candidates_respect_block_limits():
    from mfem_gb300 import autotune as at
    for (D, Q) in sorted(at.DQ3):
        for prec in at.PRECS:
            for kind in at.KINDS:
                c = at.candidates_3d(prec, D, Q, kind)
                assert c and c[0] == 1
                assert all(n * Q <= 64 and n * Q ** 3 <= 1024 for n in c)


def test_3d_kernel_list_matches_library_dispatch():
    """The tuner's DQ3 set is the library's GBPA_DQ3_LIST (= GBPA_DQ_LIST)."""
    import re
    from mfem_gb300 import autotune as at
    src = open(os.path.join(REPO, "mfem_gb300", "csrc", "gbpa_dispatch.cuh")).read()
    body = src[src.index("#define GBPA_DQ_LIST"):src.index("#define GBPA_DQ3_LIST")]
    pairs = {(int(a), int(b)) for a, b in re.findall(r"X\((\d+),\s*(\d+)\)", body)}
    assert "GBPA_DQ3_LIST(X) GBPA_DQ_LIST(X)" in src
    assert pairs == at.DQ3


def test_tensor_core_list_matches_library_dispatch():
    """The tuner's TC set is the library's GBPA_TC_LIST."""
    import re
    from mfem_gb300 import autotune as at
    src = open(os.path.join(REPO, "mfem_gb300", "csrc", "gbpa_apply_tc.cu")).read()
    line = next(ln for ln in src.splitlines() if ln.startswith("#define GBPA_TC_LIST"))
    pairs = {(int(a), int(b)) for a, b, _ in re.findall(r"X\((\d+),\s*(\d+),\s*(\d+)\)", line)}
    assert pairs == at.TC


@pytest.mark.parametrize("p", range(1, 9))
def test_element_flops_against_the_closed_form(p):
    """The bench's diffusion flop count is the kernel's contraction sequence:
    the reference's formula 2[2D^3Q + 3D^2Q^2 + 3DQ^3 + 9Q^3 + 3DQ^3 + 3D^2Q^2
    + 3D^3Q] minus the D^3 Q multiply-adds the fused backward x stage saves."""
    import bench
    D, Q = p + 1, p + 2
    ref = 2 * (2 * D ** 3 * Q + 3 * D ** 2 * Q ** 2 + 3 * D * Q ** 3 + 9 * Q ** 3 + 3 * D * Q ** 3
               + 3 * D ** 2 * Q ** 2 + 3 * D ** 3 * Q)
    assert bench.element_flops(D, Q, "diffusion") == ref - 2 * D ** 3 * Q
    mass = 2 * 2 * (D ** 3 * Q + D ** 2 * Q ** 2 + D * Q ** 3) + Q ** 3
    assert bench.element_flops(D, Q, "mass") == mass


def test_algorithmic_bytes_at_the_headline_size():
    """p=4, n=77: the element kernel's algorithmic bytes quoted in the docs."""
    import bench
    ne, D, Q = 77 ** 3, 5, 6
    ndofs = (4 * 77 + 1) ** 3
    b = bench.algorithmic_bytes(ne, ndofs, D, Q, 8, "diffusion", element_only=True)
    assert abs(b / 1e9 - 5.654) < 0.002


class _FakeLib:
    """Records the tuning calls; rejects what the library would reject."""

    def __init__(self):
        self.nbz, self.layout = {}, {}

    def gbpa_set_elements_per_block(self, kind, prec, D, Q, nbz):
        if nbz < 0 or nbz * Q * Q > 1024:
            return -1
        self.nbz[(kind, prec, D, Q)] = nbz
        return 0

    def gbpa_set_apply_layout(self, kind, prec, D, Q, layout, nbz):
        from mfem_gb300 import autotune as at
        if layout == at.GBPA_LAYOUT_TC:
            if kind != 0 or prec != 1 or (D, Q) not in at.TC:
                return -2
            self.layout[(kind, prec, D, Q)] = (layout, 0)
            return 0
        if nbz < 1 or nbz * Q > 64 or nbz * Q ** 3 > 1024:
            return -1
        self.layout[(kind, prec, D, Q)] = (layout, nbz)
        return 0


def test_load_default_installs_the_committed_table():
    from mfem_gb300 import autotune as at
    lib = _FakeLib()
    t = tuning()
    n = at.load_default(lib)
    tc = t.get("tensor_core", {})
    assert n == len(t["nbz"]) + len(t.get("layout3d", {})) + len(tc)
    assert len(lib.layout) == len(set(t.get("layout3d", {})) | set(tc))
    for k in tc:
        kind, prec, D, Q = k.split(":")
        assert lib.layout[(at.KINDS[kind], at.PRECS[prec], int(D), int(Q))] == (at.GBPA_LAYOUT_TC, 0)


def test_tensor_core_entries_name_kernels_that_exist():
    """Every committed tensor-core entry is FP32 diffusion at an order with a
    tensor-core kernel, and its recorded timing shows the tensor cores ahead
    of the CUDA cores on the same mesh."""
    from mfem_gb300 import autotune as at
    t = tuning()
    for k, v in t.get("tensor_core", {}).items():
        kind, prec, D, Q = k.split(":")
        assert kind == "diffusion" and prec == "f32" and (int(D), int(Q)) in at.TC and v == 1, k
        ms = t["tensor_core_timings"][k]["mult_ms"]
        assert ms["tensor_core"] < ms["cuda_core"], k


def test_tensor_core_section_overrides_and_is_checked(tmp_path):
    """A tensor-core entry is installed after (and so replaces) a 3D-layout
    entry for the same key; entries the library refuses (FP64, mass, an
    order without a kernel) or whose value is not 1 install nothing."""
    from mfem_gb300 import autotune as at
    lib = _FakeLib()
    f = tmp_path / "tc.json"
    f.write_text(json.dumps({"nbz": {}, "layout3d": {"diffusion:f32:5:6": 1},
                             "tensor_core": {"diffusion:f32:5:6": 1, "diffusion:f64:5:6": 1, "mass:f32:5:6": 1,
                                             "diffusion:f32:7:8": 1, "diffusion:f32:3:4": 0}}))
    n = at.load_default(lib, str(f))
    assert n == 2
    assert lib.layout == {(0, 1, 5, 6): (at.GBPA_LAYOUT_TC, 0)}


def test_load_default_tolerates_bad_files(tmp_path):
    from mfem_gb300 import autotune as at
    lib = _FakeLib()
    assert at.load_default(lib, str(tmp_path / "absent.json")) == 0
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    with pytest.warns(UserWarning):
        assert at.load_default(lib, str(bad)) == 0
    odd = tmp_path / "odd.json"
    odd.write_text(json.dumps({"nbz": {"diffusion:f64:5:6": 7, "diffusion:f64:5:6:x": 1}}))
    with pytest.warns(UserWarning):
        at.load_default(lib, str(odd))
    rejected = tmp_path / "rejected.json"
    rejected.write_text(json.dumps({"nbz": {"diffusion:f64:5:6": 500}, "layout3d": {"diffusion:f64:9:10": 2}}))
    assert at.load_default(lib, str(rejected)) == 0   # both entries refused by the library, none installed


def test_load_default_skips_only_malformed_entries(tmp_path):
    """A malformed entry is named in the warning and skipped; the valid
    entries before and after it are installed, and the count says so."""
    from mfem_gb300 import autotune as at
    lib = _FakeLib()
    mixed = tmp_path / "mixed.json"
    mixed.write_text(json.dumps({"nbz": {"diffusion:f64:5:6": 7, "diffusion:f64:bad:6": 2, "mass:f32:5:6": 3},
                                 "layout3d": {"diffusion:f64x2:5:6": 1, "nope": 1}}))
    with pytest.warns(UserWarning, match="skipped malformed entries"):
        n = at.load_default(lib, str(mixed))
    assert n == 3
    assert lib.nbz == {(0, 0, 5, 6): 7, (1, 1, 5, 6): 3}
    assert lib.layout == {(0, 2, 5, 6): (1, 1)}
    # a table that is not a JSON object installs nothing
    arr = tmp_path / "arr.json"
    arr.write_text("[1, 2]")
    lib2 = _FakeLib()
    with pytest.warns(UserWarning):
        assert at.load_default(lib2, str(arr)) == 0
    assert not lib2.nbz and not lib2.layout
