"""Failure detection without a GPU fault: each of the library's bounded device
waits is made to run out (the arrival it waits for never comes), must return
GBPA_ERR_TIMEOUT within its limit, and must leave the context usable -- the
operator apply after it gives the same result as before it."""
import time

import pytest
import torch

pytestmark = pytest.mark.gpu

GBPA_ERR_TIMEOUT = -7


def small_operator():
    from mfem_gb300 import fem
    from mfem_gb300.pa import DiffusionIntegrator, FiniteElementSpace, PAOperator
    mesh = fem.CartesianMesh(4, jitter=0.1, seed=5)
    fes = FiniteElementSpace(mesh, 3)
    integ = DiffusionIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    return PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata,
                      ess=fes.GetBoundaryTrueDofs(), precision=1)


@pytest.mark.parametrize("which,limit", [(0, 20000), (1, 2000)])
def test_bounded_wait_runs_out_and_context_stays_usable(which, limit):
    from tests.gpu_util import dev
    d = dev()
    A = small_operator()   # FP32: the TMA-staged element kernel
    gen = torch.Generator(device="cuda").manual_seed(31)
    x = torch.rand(A.ndofs, dtype=torch.float32, device="cuda", generator=gen)
    y0, y1 = torch.empty_like(x), torch.empty_like(x)
    A.Mult(x, y0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    assert d.lib.gbpa_selftest_bounded_wait(d.ctx, which, limit) == GBPA_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 10.0
    assert d.error_flags() == 0   # the timeout flag was read and cleared
    A.Mult(x, y1)
    torch.cuda.synchronize()
    assert torch.equal(y0, y1)


def test_bounded_wait_rejects_bad_arguments():
    from tests.gpu_util import dev
    d = dev()
    assert d.lib.gbpa_selftest_bounded_wait(d.ctx, 2, 100) == -1
    assert d.lib.gbpa_selftest_bounded_wait(d.ctx, 0, 0) == -1
    assert d.lib.gbpa_selftest_bounded_wait(d.ctx, 1, 1 << 27) == -1
    assert d.lib.gbpa_selftest_bounded_wait(None, 0, 100) == -1
