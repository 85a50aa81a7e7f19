"""The C-ABI libraries load and export every entry point their headers declare
(no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header: str):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*[\s\*]+([a-z][a-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_gpu_library_exports(gpu_lib):
    names = declared("se2gpu.h")
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(gpu_lib, n)]
    assert not missing, missing
    from se2dr_fork_gb300 import gpu
    assert sorted(gpu.EXPORTS) == names


def test_nn_library_exports(nn_lib):
    from se2dr_fork_gb300 import nn
    names = declared("se2nn.h")
    assert sorted(nn.EXPORTS) == names
    lib = nn_lib
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_host_library_exports():
    from se2dr_fork_gb300 import host
    names = declared("se2host.h")
    assert "se2_setup_create" in names and "se2_gaussian_random_field" in names
    lib = host.lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_gpu_library_is_sm103a(gpu_lib):
    """The library in use is the one built in the tree, for sm_103a only."""
    from se2dr_fork_gb300 import build, gpu
    path = gpu.lib_path()
    assert path.startswith(os.path.join(ROOT, "se2dr_fork_gb300"))
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert all(a in build.NVCC_FLAGS for a in build.ARCH)


def test_create_rejects_bad_problem_without_gpu(gpu_lib):
    """Argument checks run before any device call."""
    from se2dr_fork_gb300 import gpu
    h = ctypes.c_void_p()
    pr = gpu._CProblem(mx=0, my=4, p=2, dt=1e-3)
    rc = gpu.lib().se2gpu_create(ctypes.byref(pr), 64, 0, ctypes.byref(h))
    assert rc == -1 and not h.value
    assert b"positive" in gpu.lib().se2gpu_create_error()
    pr = gpu._CProblem(mx=4, my=4, p=9, dt=1e-3)
    assert gpu.lib().se2gpu_create(ctypes.byref(pr), 64, 0, ctypes.byref(h)) == -1
    pr = gpu._CProblem(mx=4, my=4, p=2, dt=1e-3)
    assert gpu.lib().se2gpu_create(ctypes.byref(pr), 16, 0, ctypes.byref(h)) == -1


def _small_problem():
    from se2dr_fork_gb300 import gpu, host, spec
    su = host.Setup(spec.demo(4, 3, p=2, tmax=1.0).replace(nt=4))
    pr, keep = gpu._problem(su)
    return su, pr, keep


@pytest.mark.parametrize("case", ["too_large", "bad_receiver", "bad_mass", "bad_source", "negative_capacity",
                                  "zero_dt", "missing_table"])
def test_create_validates_the_problem_without_gpu(gpu_lib, case):
    """Every argument check of se2gpu_create runs on the host before any device call."""
    import numpy as np
    from se2dr_fork_gb300 import gpu
    su, pr, keep = _small_problem()
    cap = 4
    if case == "too_large":            # more than 2^31 DOF: 32-bit node indices would overflow
        pr.mx, pr.my, pr.p = 30000, 30000, 8
        msg = b"too large"
    elif case == "bad_receiver":       # a receiver node that is not the named GLL point of its element
        rn = np.array(su.rec_node, dtype=np.int32)
        rn[0] += 1
        keep.append(rn)
        pr.rec_node = rn.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        msg = b"is not GLL point"
    elif case == "bad_mass":           # a non-positive lumped mass (the first one is reported)
        m = np.array(su.mass)
        m[7] = 0.0
        m[9] = -1.0
        keep.append(m)
        pr.mass = m.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        msg = b"node 7 is not positive"
    elif case == "bad_source":
        se = np.array(su.src_elem, dtype=np.int32)
        se[0] = su.mx * su.my
        keep.append(se)
        pr.src_elem = se.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        msg = b"out of range"
    elif case == "negative_capacity":
        cap = -1
        msg = b"negative"
    elif case == "zero_dt":
        pr.dt = 0.0
        msg = b"time step"
    else:
        pr.mass = None
        msg = b"missing problem table"
    h = ctypes.c_void_p()
    for precision in (64, 34, 33, 32):
        rc = gpu.lib().se2gpu_create(ctypes.byref(pr), precision, cap, ctypes.byref(h))
        assert rc == -1 and not h.value, case
        assert msg in gpu.lib().se2gpu_create_error(), gpu.lib().se2gpu_create_error()


@pytest.mark.parametrize("case", ["no_shots", "fp64", "block_zero", "block_too_long", "null_out"])
def test_ensemble_create_validates_arguments_without_gpu(gpu_lib, case):
    """The batched ensemble's argument checks run on the host before any device call."""
    from se2dr_fork_gb300 import gpu
    su, pr, keep = _small_problem()
    shots = (gpu._CProblem * 1)(pr)
    nshots, precision, block, msg = 1, 33, 100, None
    if case == "no_shots":
        nshots, msg = 0, b"at least one shot"
    elif case == "fp64":
        precision, msg = 64, b"FP32 precisions only"
    elif case == "block_zero":
        block, msg = 0, b"outside 1..4096"
    elif case == "block_too_long":
        block, msg = 4097, b"outside 1..4096"
    else:
        msg = b"null output handle"
    h = ctypes.c_void_p()
    out = None if case == "null_out" else ctypes.byref(h)
    rc = gpu.lib().se2gpu_ensemble_create(shots, nshots, precision, block, out)
    assert rc == -1 and not h.value, case
    assert msg in gpu.lib().se2gpu_ensemble_last_error(None)


@pytest.mark.parametrize("change,msg", [
    (dict(width=24), b"invalid network configuration"),       # not a multiple of 16 (tensor-core tiles)
    (dict(cin=8), b"invalid network configuration"),
    (dict(modes=65), b"invalid network configuration"),       # more modes than the grid resolves
    (dict(nout=100), b"invalid network configuration"),       # not a multiple of the grid rows
    (dict(max_batch=0), b"invalid network configuration"),
    (dict(max_batch=256), b"batch too large for the launch grid"),
])
def test_surrogate_create_validates_the_configuration_without_gpu(nn_lib, change, msg):
    """se2nn_create checks the network shape on the host before any device call."""
    import dataclasses
    from se2dr_fork_gb300 import nn
    cfg = dataclasses.replace(nn.Config(), **change).c()
    h = ctypes.c_void_p()
    assert nn.lib().se2nn_create(ctypes.byref(cfg), 0, ctypes.byref(h)) == -1 and not h.value
    assert msg in nn.lib().se2nn_last_error(None)


@pytest.mark.parametrize("n,msg", [(0, b"at least 1"), (-5, b"at least 1"),
                                   ((1 << 28) + 1, b"exceeds the scratch limit")])
def test_noalloc_norms_reject_bad_lengths_without_gpu(gpu_lib, n, msg):
    """The allocation-free norms refuse lengths outside 1..2^28 before touching the device
    (the pointers are never dereferenced on these paths)."""
    from se2dr_fork_gb300 import gpu
    out = (ctypes.c_double * 6)()
    rc = gpu.lib().se2gpu_norms_device_noalloc(ctypes.c_void_p(256), ctypes.c_void_p(512), n, None, out)
    assert rc == -1
    assert msg in gpu.lib().se2gpu_last_error(None)
    assert gpu.lib().se2gpu_norms_device_noalloc(None, ctypes.c_void_p(512), 10, None, out) == -1
    assert b"null argument" in gpu.lib().se2gpu_last_error(None)


def test_tile_configuration_queries_reject_a_null_handle_without_gpu(gpu_lib):
    """The tile-configuration entry points return SE2GPU_ERR_ARG (-1) for a null handle
    before any device call (se2gpu_tile_config included)."""
    from se2dr_fork_gb300 import gpu
    L = gpu.lib()
    info = (ctypes.c_int * 4)()
    e = (ctypes.c_int * 4)()
    assert L.se2gpu_tile_config(None) == -1
    assert L.se2gpu_set_tile_config(None, 0) == -1
    assert L.se2gpu_tile_configs(None, e, e, 4) == -1
    assert L.se2gpu_tile_config_info(None, 0, info) == -1
