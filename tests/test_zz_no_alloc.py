"""se2gpu_norms_device_noalloc: the log norms on caller-owned device vectors,
computed in a fixed static device scratch array (no device allocation),
checked through the C-ABI against se2gpu_norms on the same state.

max and min must agree exactly; the l2 norms are sums taken in a different
order, so they agree to a relative 1e-12.
"""
import ctypes as C

import numpy as np
import pytest

from se2dr_fork_gb300 import gpu as G
from se2dr_fork_gb300 import host as H
from se2dr_fork_gb300 import spec as S

pytestmark = pytest.mark.gpu

L2_RTOL = 1e-12
MAX_VALUES = 65536 * 4096   # SE2GPU_NOALLOC_MAX_VALUES


def noalloc_norms(u_ptr, v_ptr, n):
    out = np.zeros(6)
    rc = G.lib().se2gpu_norms_device_noalloc(C.c_void_p(u_ptr), C.c_void_p(v_ptr), n, None,
                                             out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0, G.lib().se2gpu_last_error(None).decode()
    return out


def check(got, ref):
    assert got[0] == ref[0] and got[1] == ref[1] and got[3] == ref[3] and got[4] == ref[4], (got, ref)
    np.testing.assert_allclose(got[[2, 5]], ref[[2, 5]], rtol=L2_RTOL, atol=0)


@pytest.mark.parametrize("mx,p", [(16, 4), (256, 4)])   # 1 block, 33 blocks of 65536 values
def test_noalloc_norms_match_se2gpu_norms_twice(gpu_lib, mx, p):
    setup = H.Setup(S.explosion64(mx, mx, p=p, tmax=1.0).replace(nt=80))
    sol = G.Solver(setup, "fp64")
    sol.advance(40)
    ref = sol.norms()
    u, v, _ = sol.device_fields()
    first = noalloc_norms(u, v, setup.ndof)
    second = noalloc_norms(u, v, setup.ndof)
    check(first, ref)
    check(second, ref)
    assert np.array_equal(first, second)
    sol.advance(40)
    ref = sol.norms()
    u, v, _ = sol.device_fields()
    check(noalloc_norms(u, v, setup.ndof), ref)
    assert ref[2] > 0 and ref[5] > 0


def test_noalloc_norms_rejects_sizes_beyond_the_scratch(gpu_lib):
    setup = H.Setup(S.explosion64(8, 8, p=2, tmax=1.0).replace(nt=4))
    sol = G.Solver(setup, "fp64")
    u, v, _ = sol.device_fields()
    out = np.zeros(6)
    rc = G.lib().se2gpu_norms_device_noalloc(C.c_void_p(u), C.c_void_p(v), MAX_VALUES + 1, None,
                                             out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == -1
    assert b"scratch limit" in G.lib().se2gpu_last_error(None)
    rc = G.lib().se2gpu_norms_device_noalloc(C.c_void_p(u), C.c_void_p(v), 0, None,
                                             out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == -1
