"""In-tree build of the native libraries.

* ``lib/libse2host.so``  -- FP64 host set-up (C, gcc), include/se2host.h
* ``lib/libse2gpu.so``   -- sm_103a kernels + C-ABI (nvcc), include/se2gpu.h
* ``lib/libse2nn.so``    -- the surrogate network runtime (nvcc), include/se2nn.h
* ``bin/se2wave_gpu``    -- the C host application (se2wave's command line)

Each translation unit is compiled in parallel and only when its sources are
newer than its object.  Host C/C++ is compiled with -ffp-contract=off: the FP64
set-up must round every product and sum separately, like the reference.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")
OBJ = os.path.join(PKG, "_build")

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
CC = os.environ.get("CC", "gcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INC}"]
CC_FLAGS = ["-O2", "-std=gnu99", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", f"-I{INC}"]

CU_UNITS = ["se2gpu_f64", "se2gpu_f32", "se2gpu_f32p", "se2gpu_f32df", "se2gpu_api", "se2gpu_ensemble", "se2gpu_noalloc", "se2gpu_peaks"]
CU_DEPS = ["se2gpu_kernels.cuh", "se2gpu_launch.h", "se2gpu_persist.cuh", "se2gpu_persist_launch.h", "se2gpu_persist_params.h", "se2gpu_internal.h"]


def _newer(target: str, sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_host(force: bool = False) -> str:
    os.makedirs(LIB, exist_ok=True)
    out = os.path.join(LIB, "libse2host.so")
    src = os.path.join(CSRC, "se2_host.c")
    if force or _newer(out, [src, os.path.join(INC, "se2host.h")]):
        _run([CC, *CC_FLAGS, "-shared", "-o", out, src, "-lm"])
    return out


NN_UNITS = ["se2nn"]
NN_DEPS = ["se2nn_gemm.cuh", "se2nn_tc.cuh"]


def build_gpu(force: bool = False) -> str:
    return _build_cuda_lib("libse2gpu.so", CU_UNITS, [os.path.join(CSRC, d) for d in CU_DEPS] + [os.path.join(INC, "se2gpu.h")], force)


def build_nn(force: bool = False) -> str:
    return _build_cuda_lib("libse2nn.so", NN_UNITS, [os.path.join(CSRC, d) for d in NN_DEPS] + [os.path.join(INC, "se2nn.h")], force)


def _build_cuda_lib(name: str, units, deps, force: bool) -> str:
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    out = os.path.join(LIB, name)
    jobs = []
    objs = []
    for u in units:
        src = os.path.join(CSRC, u + ".cu")
        obj = os.path.join(OBJ, u + ".o")
        objs.append(obj)
        if force or _newer(obj, [src, *deps]):
            jobs.append([NVCC, *NVCC_FLAGS, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _newer(out, objs):
        _run([NVCC, *ARCH, "-shared", "-o", out, *objs, "-lcudart", "-lpthread"])
    return out


def build_app(force: bool = False) -> str:
    os.makedirs(BIN, exist_ok=True)
    out = os.path.join(BIN, "se2wave_gpu")
    src = os.path.join(CSRC, "se2wave_gpu.c")
    if not os.path.exists(src):
        return ""
    libs = [os.path.join(LIB, "libse2host.so"), os.path.join(LIB, "libse2gpu.so")]
    if force or _newer(out, [src, *libs, os.path.join(INC, "se2gpu.h"), os.path.join(INC, "se2host.h")]):
        _run([CC, *[f for f in CC_FLAGS if f != "-fPIC"], "-o", out, src, f"-L{LIB}", "-lse2gpu", "-lse2host", "-lm",
              f"-Wl,-rpath,{LIB}"])
    return out


def build_all(force: bool = False) -> dict:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        fh = ex.submit(build_host, force)
        fg = ex.submit(build_gpu, force)
        fn = ex.submit(build_nn, force)
        host, gpu, nn = fh.result(), fg.result(), fn.result()
    app = build_app(force)
    return {"host": host, "gpu": gpu, "nn": nn, "app": app}


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
