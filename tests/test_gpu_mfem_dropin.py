"""MFEM itself calling libgbpa: the cfg1 program written against MFEM's
unchanged API (integration/ex1_gbpa.cpp: BilinearForm with
SetAssemblyLevel(AssemblyLevel::PARTIAL), FormLinearSystem, CGSolver +
OperatorJacobiSmoother), linked to the reference MFEM build whose
PABilinearFormExtension carries the libgbpa hooks (integration/
mfem_gbpa_patch.py). With MFEM_GBPA=1 every operator Mult of the solve runs in
libgbpa on the GPU (gbpa_operator_create_host from MFEM's own restriction maps,
basis tables and PA data; gbpa_operator_mult_host on MFEM's host Vectors).
The solution must match the reference's golden cfg1 solve to the PCG bar
(1e-10 relative L2) with the same iteration count (+-1), every CG Mult must
have been forwarded, and libgbpa.so must be mapped into the MFEM process."""
import json
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import REPO, load_golden

pytestmark = pytest.mark.gpu


def test_mfem_cfg1_solve_through_libgbpa(tmp_path):
    import __graft_entry__ as ge
    exe = os.path.join(ge.dropin_dir(), "ex1_gbpa")
    if not os.path.exists(exe):
        pytest.skip("the MFEM drop-in is built by build() where the reference sources are staged")
    out = tmp_path / "x.bin"
    env = dict(os.environ, MFEM_GBPA="1")
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    info = json.loads(r.stdout.strip().splitlines()[-1])
    print(json.dumps(info))
    g = load_golden("cfg1_solve")
    x = np.fromfile(out)
    assert info["converged"] == 1
    assert abs(info["iterations"] - int(g["cg_info"][0])) <= 1
    # the CG's operator applications (one per iteration, plus the initial
    # residual) all went through libgbpa
    assert info["forwarded_mults"] >= info["iterations"]
    assert info["libgbpa_mapped"].endswith("libgbpa.so")
    assert os.path.realpath(info["libgbpa_mapped"]).startswith(os.path.realpath(REPO))
    rel = np.linalg.norm(x - g["X"]) / np.linalg.norm(g["X"])
    print(f"rel_l2_vs_reference_cfg1 {rel:.3e}")
    assert rel < 1e-10
