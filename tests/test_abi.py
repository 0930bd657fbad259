"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares; the Python binding declares exactly that set; the host
map construction (an ABI entry that needs no GPU) is bit-identical to the
reference's maps."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from tests.conftest import REPO, golden_cases, load_golden


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(gbpa_\w+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from mfem_gb300 import _lib
    return _lib.load()


def test_header_declares_entry_points():
    assert len(declared_symbols()) >= 30


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_matches_header():
    from mfem_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == declared_symbols()


def _prototypes():
    """name -> (return type, [parameter types]) parsed from include/*.h."""
    protos = {}
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"([A-Za-z_][\w \t\*]*?)\b(gbpa_\w+)\s*\(([^)]*)\)\s*;", src):
            ret = " ".join(m.group(1).split())
            params = []
            for a in m.group(3).split(","):
                a = " ".join(a.split())
                if not a or a == "void":
                    continue
                params.append(a if a.endswith("*") else re.sub(r"\s*\b\w+$", "", a))
            protos[m.group(2)] = (ret, params)
    return protos


def _c_kind(t):
    """Type class of a C type: pointers and library handles are 'p'."""
    t = t.replace("const ", "").strip()
    if "*" in t or (t.startswith("gbpa_") and t.endswith("_t")):
        return "p"
    return {"int": "i4", "int64_t": "i8", "long long": "i8", "unsigned long long": "u8",
            "double": "f8", "float": "f4", "void": "v"}[t]


def _ctypes_kind(t):
    if t is None:
        return "v"
    if t in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(t, "_type_") and isinstance(t._type_, type):
        return "p"
    if t is ctypes.c_double:
        return "f8"
    if t is ctypes.c_float:
        return "f4"
    unsigned = t in (ctypes.c_uint, ctypes.c_uint64, ctypes.c_ulonglong, ctypes.c_ulong)
    return ("u" if unsigned else "i") + str(ctypes.sizeof(t))


def test_binding_argument_types_match_header():
    """Every prototype's return and parameter types agree with the ctypes
    signature the binding gives the library (count, and pointer / int /
    64-bit int / double class of each)."""
    from mfem_gb300 import _lib
    protos = _prototypes()
    assert sorted(protos) == declared_symbols()
    bad = []
    for name, (ret, params) in protos.items():
        res, args = _lib.SIGNATURES[name]
        want = [_c_kind(t) for t in params]
        have = [_ctypes_kind(t) for t in args]
        if want != have or _c_kind(ret) != _ctypes_kind(res):
            bad.append((name, ret, want, _ctypes_kind(res), have))
    assert not bad, bad


def test_version_and_error_strings(lib):
    assert lib.gbpa_version() == 10000
    assert lib.gbpa_error_string(0) == b"success"
    assert b"invalid" in lib.gbpa_error_string(-1)


def test_null_arguments_are_rejected_without_gpu(lib):
    # argument validation happens before any CUDA call
    assert lib.gbpa_diffusion_apply3d(None, 1, 1, 3, 4, None, None, None, None, None, None, None) == -1
    assert lib.gbpa_operator_create(None, None, None) == -1
    assert lib.gbpa_restriction_build(-1, 8, 1, None, None, None, None, None) == -1


@pytest.mark.parametrize("case", golden_cases())
def test_host_restriction_build_bit_exact(lib, case):
    g = load_golden(case)
    ne, ndofs, D = (int(v) for v in g["meta"][:3])
    nd = D ** 3
    off = np.zeros(ndofs + 1, np.int32); ind = np.zeros(ne * nd, np.int32); gm = np.zeros(ne * nd, np.int32)
    ed = np.ascontiguousarray(g["elem_dofs"], np.int32); dm = np.ascontiguousarray(g["dof_map"], np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.gbpa_restriction_build(ne, nd, ndofs, P(ed), P(dm), P(off), P(ind), P(gm)) == 0
    assert np.array_equal(gm, g["gather_map"])
    assert np.array_equal(off, g["offsets"])
    assert np.array_equal(ind, g["indices"])


def test_host_restriction_build_rejects_out_of_range(lib):
    ed = np.array([0, 1, 2, 99], np.int32)
    off = np.zeros(5, np.int32); ind = np.zeros(4, np.int32); gm = np.zeros(4, np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.gbpa_restriction_build(1, 4, 4, P(ed), None, P(off), P(ind), P(gm)) == -9


def test_block_layout_switch_without_gpu(lib):
    """The FP32 block apply's kernel choice is host state: the tensor-core
    block kernel by default where one exists ((5,6) and (6,7), 8 vectors),
    the CUDA-core kernel elsewhere; TC is refused where no kernel exists and
    any other layout is an invalid argument."""
    TC = 2
    assert lib.gbpa_get_block_apply_layout(6, 7, 8) == TC
    assert lib.gbpa_get_block_apply_layout(5, 6, 8) == TC
    assert lib.gbpa_get_block_apply_layout(4, 5, 8) == 0
    assert lib.gbpa_get_block_apply_layout(6, 7, 2) == 0
    assert lib.gbpa_set_block_apply_layout(4, 5, 8, TC) == -2
    assert lib.gbpa_set_block_apply_layout(6, 7, 8, 1) == -1
    assert lib.gbpa_set_block_apply_layout(6, 7, 0, 0) == -1
    assert lib.gbpa_get_block_apply_layout(17, 18, 8) == -1
    assert lib.gbpa_set_block_apply_layout(6, 7, 8, 0) == 0
    try:
        assert lib.gbpa_get_block_apply_layout(6, 7, 8) == 0
    finally:
        assert lib.gbpa_set_block_apply_layout(6, 7, 8, TC) == 0
    assert lib.gbpa_get_block_apply_layout(6, 7, 8) == TC


def test_host_operator_create_rejects_bad_arguments_without_gpu(lib):
    """gbpa_operator_create_host validates before touching the GPU: no
    context or descriptor, bad kind or precision, negative sizes, and a
    missing array are all GBPA_ERR_INVALID_ARGUMENT."""
    import ctypes
    from mfem_gb300 import _lib
    op = ctypes.c_void_p()
    assert lib.gbpa_operator_create_host(None, None, ctypes.byref(op)) == -1
    d = _lib.OperatorDesc(0, 0, 1, 8, 2, 3, 1, None, None, None, None, None, None, None, 0, 0)
    fake_ctx = ctypes.c_void_p(1)   # never dereferenced: the descriptor is refused first
    assert lib.gbpa_operator_create_host(fake_ctx, ctypes.byref(d), ctypes.byref(op)) == -1   # arrays missing
    for field, value in (("kind", 7), ("precision", 9), ("ne", -1), ("d1d", 0)):
        bad = _lib.OperatorDesc(0, 0, 1, 8, 2, 3, 1, None, None, None, None, None, None, None, 0, 0)
        setattr(bad, field, value)
        assert lib.gbpa_operator_create_host(fake_ctx, ctypes.byref(bad), ctypes.byref(op)) == -1, field
