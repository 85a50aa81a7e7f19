"""ctypes binding of the surrogate network runtime (include/se2nn.h, lib/libse2nn.so).

Device memory for inputs, targets and outputs is held in torch tensors (plain
device buffers); every computation on them is a kernel of libse2nn.so.  There
is no CPU fallback: construction raises when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import Optional

import numpy as np

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libse2nn.so")
_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
vp = C.c_void_p

EXPORTS = ["se2nn_create", "se2nn_destroy", "se2nn_last_error", "se2nn_set_stream", "se2nn_num_params",
           "se2nn_get_params", "se2nn_set_params", "se2nn_get_grads", "se2nn_set_receivers", "se2nn_forward",
           "se2nn_loss_grad", "se2nn_adam_step", "se2nn_build_inputs", "se2nn_gather_targets", "se2nn_gemm",
           "se2nn_set_tensor_path", "se2nn_tensor_path_info"]


class CConfig(C.Structure):
    _fields_ = [("ny", C.c_int), ("nx", C.c_int), ("cin", C.c_int), ("width", C.c_int), ("modes", C.c_int),
                ("layers", C.c_int), ("nrec", C.c_int), ("nout", C.c_int), ("hidden", C.c_int),
                ("max_batch", C.c_int)]


@dataclasses.dataclass
class Config:
    """Network shape; the defaults are the 128^2, width-64, 16-mode, 4-layer operator
    producing 16 receivers x 128 rows x 16 values (2 components x 1024 samples)."""
    ny: int = 128
    nx: int = 128
    cin: int = 16
    width: int = 64
    modes: int = 16
    layers: int = 4
    nrec: int = 16
    nout: int = 2048
    hidden: int = 128
    max_batch: int = 32

    def c(self) -> CConfig:
        return CConfig(*[getattr(self, f.name) for f in dataclasses.fields(self)])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise RuntimeError(f"{_LIB_PATH} is missing: the CUDA library must be built (__graft_entry__.build())")
        L = C.CDLL(_LIB_PATH)
        L.se2nn_create.argtypes = [C.POINTER(CConfig), C.c_ulonglong, C.POINTER(vp)]
        L.se2nn_destroy.argtypes = [vp]
        L.se2nn_destroy.restype = None
        L.se2nn_last_error.argtypes = [vp]
        L.se2nn_last_error.restype = C.c_char_p
        L.se2nn_set_stream.argtypes = [vp, vp]
        L.se2nn_num_params.argtypes = [vp]
        L.se2nn_num_params.restype = C.c_long
        L.se2nn_get_params.argtypes = [vp, _fp]
        L.se2nn_set_params.argtypes = [vp, _fp]
        L.se2nn_get_grads.argtypes = [vp, _fp]
        L.se2nn_set_receivers.argtypes = [vp, _ip]
        L.se2nn_forward.argtypes = [vp, vp, C.c_int, vp]
        L.se2nn_loss_grad.argtypes = [vp, vp, C.c_int, vp, _dp, vp]
        L.se2nn_adam_step.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]
        L.se2nn_build_inputs.argtypes = [vp, vp, vp, vp, C.c_int, C.c_float, vp]
        L.se2nn_gather_targets.argtypes = [vp, vp, vp, C.c_int, vp]
        L.se2nn_gemm.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_long, C.c_long, C.c_long,
                                 C.c_long, C.c_long, C.c_long, C.c_int, C.c_int, C.c_float, C.c_float, vp]
        L.se2nn_set_tensor_path.argtypes = [C.c_int]
        L.se2nn_tensor_path_info.argtypes = [C.POINTER(C.c_long)]
        _lib = L
    return _lib


class NnError(RuntimeError):
    pass


def set_tensor_path(mode: int):
    """Which GEMMs run on the tcgen05 tensor-core kernel (process-wide): 0 none (every GEMM on
    the mma.sync kernel), 1 the row GEMMs except the 1x1 convolutions' shape (N <= 64,
    32 < K <= 64), where mma.sync measured faster (default), 2 every qualifying row GEMM."""
    if lib().se2nn_set_tensor_path(int(mode)) != 0:
        raise NnError(f"tensor path mode {mode} is not 0, 1 or 2")


def tensor_path_info() -> dict:
    """GEMM launches so far by kernel, and whether a tcgen05 GEMM's bounded wait expired."""
    out = (C.c_long * 3)()
    if lib().se2nn_tensor_path_info(out) != 0:
        raise NnError("se2nn_tensor_path_info failed")
    return {"tcgen05_launches": int(out[0]), "mma_sync_launches": int(out[1]), "wait_expired": bool(out[2])}


def _ptr(t) -> int:
    return 0 if t is None else int(t.data_ptr())


def gemm(A, B, Cout, M, N, K, batch=1, lda=None, ldb=None, ldc=None, sA=0, sB=0, sC=0, transA=0, transB=0,
         alpha=1.0, beta=0.0, stream=None):
    """The network's strided-batched BF16 GEMM on torch device tensors (A, B bf16; Cout fp32)."""
    lda = (M if transA else K) if lda is None else lda
    ldb = (K if transB else N) if ldb is None else ldb
    ldc = N if ldc is None else ldc
    rc = lib().se2nn_gemm(vp(_ptr(A)), vp(_ptr(B)), vp(_ptr(Cout)), M, N, K, batch, lda, ldb, ldc, sA, sB, sC,
                          transA, transB, alpha, beta, vp(stream or 0))
    if rc != 0:
        raise NnError(lib().se2nn_last_error(None).decode())


class Network:
    """One surrogate network (parameters, Adam state, activation buffers) on the current GPU."""

    def __init__(self, cfg: Optional[Config] = None, seed: int = 0):
        self.cfg = cfg or Config()
        h = vp()
        if lib().se2nn_create(C.byref(self.cfg.c()), seed, C.byref(h)) != 0:
            raise NnError("se2nn_create: " + lib().se2nn_last_error(None).decode())
        self._h = h
        self.nparams = int(lib().se2nn_num_params(h))

    def _check(self, rc, what):
        if rc != 0:
            raise NnError(f"{what} failed ({rc}): {lib().se2nn_last_error(self._h).decode()}")

    def close(self):
        if getattr(self, "_h", None):
            lib().se2nn_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_stream(self, stream_ptr: int):
        self._check(lib().se2nn_set_stream(self._h, vp(stream_ptr)), "se2nn_set_stream")

    def params(self) -> np.ndarray:
        p = np.zeros(self.nparams, dtype=np.float32)
        self._check(lib().se2nn_get_params(self._h, p.ctypes.data_as(_fp)), "se2nn_get_params")
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        self._check(lib().se2nn_set_params(self._h, p.ctypes.data_as(_fp)), "se2nn_set_params")

    def grads(self) -> np.ndarray:
        g = np.zeros(self.nparams, dtype=np.float32)
        self._check(lib().se2nn_get_grads(self._h, g.ctypes.data_as(_fp)), "se2nn_get_grads")
        return g

    def set_receivers(self, rec_x):
        r = np.ascontiguousarray(rec_x, dtype=np.int32)
        self._check(lib().se2nn_set_receivers(self._h, r.ctypes.data_as(_ip)), "se2nn_set_receivers")
        self.rec_x = r.copy()

    def forward(self, x, out):
        """out[b] (fp32 torch tensor [B, nrec, nout]) = network(x[b]) (bf16 torch tensor [B, ny, nx, cin])."""
        self._check(lib().se2nn_forward(self._h, vp(_ptr(x)), int(x.shape[0]), vp(_ptr(out))), "se2nn_forward")

    def loss_grad(self, x, target, out=None) -> float:
        loss = C.c_double()
        self._check(lib().se2nn_loss_grad(self._h, vp(_ptr(x)), int(x.shape[0]), vp(_ptr(target)), C.byref(loss),
                                          vp(_ptr(out))), "se2nn_loss_grad")
        return loss.value

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self._check(lib().se2nn_adam_step(self._h, lr, beta1, beta2, eps, weight_decay), "se2nn_adam_step")

    def build_inputs(self, materials, src, idx, sigma_cells, x):
        self._check(lib().se2nn_build_inputs(self._h, vp(_ptr(materials)), vp(_ptr(src)), vp(_ptr(idx)),
                                             int(idx.shape[0]), float(sigma_cells), vp(_ptr(x))),
                    "se2nn_build_inputs")

    def gather_targets(self, targets, idx, out):
        self._check(lib().se2nn_gather_targets(self._h, vp(_ptr(targets)), vp(_ptr(idx)), int(idx.shape[0]),
                                               vp(_ptr(out))), "se2nn_gather_targets")
