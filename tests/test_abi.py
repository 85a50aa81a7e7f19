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
    """The library carries sm_103a device code and is the one in the tree."""
    from se2dr_fork_gb300 import gpu
    path = gpu.lib_path()
    assert path.startswith(os.path.join(ROOT, "se2dr_fork_gb300"))
    blob = open(path, "rb").read()
    assert b"sm_103a" in blob


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
