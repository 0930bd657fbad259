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
