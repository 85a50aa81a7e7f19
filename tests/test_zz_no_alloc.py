"""se2gpu_norms_device_noalloc: the log norms on caller-owned device vectors,
computed in a fixed static device scratch array (no device allocation),
checked through the C-ABI against se2gpu_norms on the same state.

max and min must agree exactly; the l2 norms are sums taken in a different
order, so they agree to a relative 1e-12.  A length that is not a multiple of
the per-block chunk is also checked against numpy on values uploaded through an
FP64 handle's fields (an all-negative vector tests the starting value of the
maximum), and a NaN in the uploaded values must fail the call as a numeric error.
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


CHUNK = 65536   # SE2GPU_NOALLOC_CHUNK


def _fp64_handle_with_fields(u, v):
    """An FP64 handle whose device u, v hold the given host vectors (the FP64 device
    layout is the reference's packed Vec layout, so set_fields copies them unchanged)."""
    setup = H.Setup(S.explosion64(128, 128, p=2, tmax=1.0).replace(nt=4))   # 257^2 nodes, 132098 values
    sol = G.Solver(setup, "fp64")
    n = setup.ndof
    uu = np.zeros(n); vv = np.zeros(n)
    uu[:u.size] = u; vv[:v.size] = v
    sol.set_fields(uu, vv, np.zeros(n))
    return sol


def test_noalloc_norms_ragged_length_against_numpy(gpu_lib):
    n = 2 * CHUNK + 17   # two full chunks and a ragged third block
    rng = np.random.default_rng(11)
    u = rng.standard_normal(n) * 3.0
    v = -np.abs(rng.standard_normal(n)) - 0.5   # all negative: max must not be the start value
    sol = _fp64_handle_with_fields(u, v)
    du, dv, _ = sol.device_fields()
    for _ in range(2):
        got = noalloc_norms(du, dv, n)
        assert got[0] == u.max() and got[1] == u.min(), got
        assert got[3] == v.max() and got[4] == v.min(), got
        assert got[3] < 0
        np.testing.assert_allclose(got[[2, 5]], [np.linalg.norm(u), np.linalg.norm(v)], rtol=L2_RTOL, atol=0)


def test_noalloc_norms_report_a_nan_as_a_numeric_error(gpu_lib):
    n = CHUNK + 5
    u = np.linspace(-1.0, 1.0, n)
    v = np.ones(n)
    u[CHUNK + 2] = np.nan   # in the ragged last block
    sol = _fp64_handle_with_fields(u, v)
    du, dv, _ = sol.device_fields()
    out = np.zeros(6)
    rc = G.lib().se2gpu_norms_device_noalloc(C.c_void_p(du), C.c_void_p(dv), n, None,
                                             out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == -5   # SE2GPU_ERR_NUMERIC
    assert b"non-finite" in G.lib().se2gpu_last_error(None)
    # the next call on finite values succeeds
    u[CHUNK + 2] = 0.5
    sol.set_fields(np.concatenate([u, np.zeros(sol.setup.ndof - n)]), np.concatenate([v, np.zeros(sol.setup.ndof - n)]),
                   np.zeros(sol.setup.ndof))
    got = noalloc_norms(du, dv, n)
    assert got[0] == 1.0 and got[1] == -1.0
