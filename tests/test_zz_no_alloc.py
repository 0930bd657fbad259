"""The allocation-free L-vector diffusion apply (gbpa_diffusion_mult_noalloc).

It serves callers that cannot allocate device memory -- an application whose
device memory belongs to its own pool allocator, or a path that must not
trigger the device synchronisation cudaMalloc/cudaFree can cause. Its scratch
E-vector is a fixed static device array shared by every call. Two calls in a
row, with different inputs, must each match the allocating fused operator
(gbpa_operator_mult) within the FP64 tolerance used throughout the tests
(1e-12 relative L2); a problem larger than the fixed scratch is refused.

The cases cover both thread layouts that write the static scratch: p = 3 (the
2D-slab kernel) and p = 6 (FP64 p >= 5 runs the 3D-layout kernel), on the
legacy default stream and on a separate torch stream.

This file is collected last so that a run stopping at the first failure has
run every other test; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest
import torch

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _noalloc(lib, stream, ne, ndofs, D, Q, B, G, qd, R, x, y):
    return lib.gbpa_diffusion_mult_noalloc(stream, ne, ndofs, D, Q, 1, _ptr(B), _ptr(G), _ptr(qd),
                                           _ptr(R.gather_map), _ptr(R.offsets), _ptr(R.indices),
                                           _ptr(x), _ptr(y))


@pytest.mark.parametrize("case", ["jit3_p3_fn", "jit2_p6_fn"])
@pytest.mark.parametrize("own_stream", [False, True])
def test_noalloc_matches_operator_two_calls(case, own_stream):
    from mfem_gb300.pa import ElementRestriction, PAOperator
    from tests.gpu_util import T, H, dev
    d = dev()
    g = load_golden(case)
    ne, ndofs, D, Q = (int(v) for v in g["meta"][:4])
    R = ElementRestriction.from_maps(ne, D ** 3, ndofs, g["gather_map"], g["offsets"], g["indices"])
    B, G, qd = T(g["B"]), T(g["G"]), T(g["qdata_diff"])
    op = PAOperator(0, R, D, Q, B, G, qd)
    rng = np.random.default_rng(7)
    xs = [T(g["x"]), T(rng.uniform(-1, 1, ndofs))]
    s = torch.cuda.Stream() if own_stream else None
    for x in xs:
        y_ref = torch.empty_like(x)
        op.Mult(x, y_ref)
        y = torch.full_like(x, float("nan"))
        torch.cuda.synchronize()
        handle = ctypes.c_void_p(s.cuda_stream) if s is not None else None
        assert _noalloc(d.lib, handle, ne, ndofs, D, Q, B, G, qd, R, x, y) == 0
        torch.cuda.synchronize()
        ref = H(y_ref)
        assert np.linalg.norm(H(y) - ref) / np.linalg.norm(ref) < 1e-12
    # and against the reference's own BilinearForm::Mult output
    y = torch.empty_like(xs[0])
    assert _noalloc(d.lib, None, ne, ndofs, D, Q, B, G, qd, R, xs[0], y) == 0
    torch.cuda.synchronize()
    assert np.linalg.norm(H(y) - g["y_diff"]) / np.linalg.norm(g["y_diff"]) < 1e-12


def test_noalloc_rejects_oversize():
    from tests.gpu_util import dev
    d = dev()
    too_many = (1 << 21) // 64 + 1     # elements of D = 4 beyond the fixed scratch
    st = d.lib.gbpa_diffusion_mult_noalloc(None, too_many, 1000, 4, 5, 1, None, None, None, None,
                                           None, None, None, None)
    assert st == -2
    # (D, Q) beyond the kernels' 16 points: unsupported, as for the other entry points
    st = d.lib.gbpa_diffusion_mult_noalloc(None, 1, 1000, 17, 18, 1, None, None, None, None,
                                           None, None, None, None)
    assert st == -2
    st = d.lib.gbpa_diffusion_mult_noalloc(None, 1, 1000, 0, 2, 1, None, None, None, None,
                                           None, None, None, None)
    assert st == -1
