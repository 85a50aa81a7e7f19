"""Failure detection of the FP32 step kernels, without a GPU fault.

Every wait of the persistent step kernels on their tile copies is bounded: on expiry
the kernel raises the handle's error flag and returns, and the host reports it.  The
self-test entry point runs that same bounded wait on an mbarrier that nothing arrives
at (256 polls), so the wait runs out on purpose while no copy is in flight.  The test
checks the status and message the host reads, that the failed handle stays failed,
and that the CUDA context is still usable: a new handle reproduces a run made before.
"""
import numpy as np
import pytest

from se2dr_fork_gb300 import gpu as G
from se2dr_fork_gb300 import host as H
from se2dr_fork_gb300 import spec as S

pytestmark = pytest.mark.gpu

SE2GPU_ERR_CUDA = -2
PRODUCTION_POLLS, TEST_POLLS = 1 << 18, 256   # WAIT_LIMIT of the step kernels, the self-test's limit


@pytest.fixture(scope="module", autouse=True)
def _lib(gpu_lib):
    return gpu_lib


def test_bounded_wait_expiry_is_reported_and_context_survives():
    setup = H.Setup(S.explosion64(12, 10, p=4, tmax=1.0).replace(nt=30))
    before = G.Solver(setup, "fp32_kahan").run()

    bad = G.Solver(setup, "fp32_kahan")
    bad.advance(10)
    rc, seconds, msg = bad.selftest_wait_expiry()
    assert rc == SE2GPU_ERR_CUDA, (rc, msg)
    assert "bounded wait expired" in msg
    assert 0.0 < seconds < 10.0
    # the step kernels' limit bounds a wait at PRODUCTION_POLLS / TEST_POLLS times this:
    # about a second, so a wait that never ends stops within seconds, not minutes
    bound = seconds * PRODUCTION_POLLS / TEST_POLLS
    print(f"{TEST_POLLS} polls of an incomplete mbarrier: {seconds * 1e6:.1f} us; "
          f"the step kernels' limit of {PRODUCTION_POLLS} polls: {bound:.2f} s")
    assert bound < 5.0
    # the flag stays raised: the handle's state is not trusted after an expiry
    bad.advance(5)
    with pytest.raises(G.GpuError, match="bounded wait expired"):
        bad.traces()
    with pytest.raises(G.GpuError, match="bounded wait expired"):
        bad.synchronize()
    bad.close()

    after = G.Solver(setup, "fp32_kahan").run()
    assert np.array_equal(before, after)
