"""The MFEM drop-in (integration/): the patch, and MFEM's own cfg1 program
with the libgbpa hooks compiled in but forwarding off (MFEM's path, no GPU).
The GPU run with forwarding on is tests/test_gpu_mfem_dropin.py."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from tests.conftest import REPO, load_golden

STAGED = os.path.join(REPO, "baseline", "_ref", "src")


def _patcher():
    sys.path.insert(0, os.path.join(REPO, "integration"))
    try:
        import mfem_gbpa_patch
    finally:
        sys.path.pop(0)
    return mfem_gbpa_patch


def test_patch_refuses_a_missing_anchor(tmp_path):
    mp = _patcher()
    (tmp_path / "fem").mkdir()
    (tmp_path / "fem" / "bilinearform_ext.cpp").write_text("// not MFEM\n")
    with pytest.raises(SystemExit, match="anchor found 0 times"):
        mp.patched((tmp_path / "fem" / "bilinearform_ext.cpp").read_text())


def test_committed_patch_is_the_patchers_diff():
    """integration/mfem_gbpa.patch is exactly what mfem_gbpa_patch.py does to
    the staged reference file (checked where the sources are staged)."""
    if not os.path.exists(os.path.join(STAGED, "fem", "bilinearform_ext.cpp")):
        pytest.skip("reference sources not staged (oracle/ref/stage_reference.py)")
    mp = _patcher()
    with open(os.path.join(REPO, "integration", "mfem_gbpa.patch")) as f:
        assert f.read() == mp.diff(STAGED)


def _driver():
    import __graft_entry__ as ge
    exe = os.path.join(ge.dropin_dir(), "ex1_gbpa")
    if not os.path.exists(exe):
        pytest.skip("the MFEM drop-in is built by build() where the reference sources are staged")
    return exe


def test_dropin_driver_without_forwarding_is_mfems_cfg1(tmp_path):
    """With forwarding off the patched MFEM runs its own PA path: the cfg1
    solution equals the reference's golden one (bit for bit on the machine the
    golden vectors were made on; 1e-12 where the compiler contracts
    multiply-adds differently, e.g. aarch64), no Mult is forwarded."""
    exe = _driver()
    out = tmp_path / "x.bin"
    env = dict(os.environ, MFEM_GBPA="0", OMP_NUM_THREADS="1")
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr
    info = json.loads(r.stdout.strip().splitlines()[-1])
    g = load_golden("cfg1_solve")
    x = np.fromfile(out)
    assert info["forwarded_mults"] == 0
    assert info["iterations"] == int(g["cg_info"][0])
    assert np.linalg.norm(x - g["X"]) / np.linalg.norm(g["X"]) < 1e-12
