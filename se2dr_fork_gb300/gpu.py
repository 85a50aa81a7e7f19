"""ctypes binding of the GB300 time-loop library (include/se2gpu.h, lib/libse2gpu.so).

This is the only compute path of the package: there is no CPU fallback.  If the
library is missing or no GPU is present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .host import Setup

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libse2gpu.so")
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

FP64, FP32_DF, FP32_KAHAN, FP32 = 64, 34, 33, 32
PRECISIONS = {"fp64": FP64, "fp32_df": FP32_DF, "fp32_kahan": FP32_KAHAN, "fp32": FP32}

# symbols declared in include/se2gpu.h
EXPORTS = ["se2gpu_create", "se2gpu_destroy", "se2gpu_last_error", "se2gpu_create_error", "se2gpu_set_stream",
           "se2gpu_synchronize", "se2gpu_selftest_wait_expiry", "se2gpu_set_fields", "se2gpu_get_fields", "se2gpu_advance", "se2gpu_traces",
           "se2gpu_norms", "se2gpu_assemble_linear_form", "se2gpu_assemble_linear_form_device", "se2gpu_info",
           "se2gpu_device_fields", "se2gpu_tile_configs", "se2gpu_tile_config_info", "se2gpu_set_tile_config",
           "se2gpu_tile_config",
           "se2gpu_ensemble_create", "se2gpu_ensemble_destroy", "se2gpu_ensemble_last_error",
           "se2gpu_ensemble_set_stream", "se2gpu_ensemble_set_graphs", "se2gpu_ensemble_set_tile_config",
           "se2gpu_ensemble_tile_config", "se2gpu_ensemble_advance", "se2gpu_ensemble_enqueue",
           "se2gpu_ensemble_synchronize", "se2gpu_ensemble_get_fields", "se2gpu_ensemble_set_fields",
           "se2gpu_ensemble_info", "se2gpu_norms_device_noalloc",
           "se2gpu_checkpoint_size", "se2gpu_checkpoint_save", "se2gpu_checkpoint_load", "se2gpu_pipe_peak"]


class _CProblem(C.Structure):
    _fields_ = [("mx", C.c_int), ("my", C.c_int), ("p", C.c_int), ("dt", C.c_double),
                ("D", _dp), ("wq", _dp), ("w1d", _dp), ("J00", _dp), ("J11", _dp), ("iJ00", _dp), ("iJ11", _dp),
                ("lambda_", _dp), ("mu", _dp), ("mass", _dp),
                ("nsrc", C.c_int), ("src_elem", _ip), ("src_vals", _dp),
                ("nrec", C.c_int), ("rec_node", _ip), ("rec_elem", _ip), ("rec_gll", _ip)]


_lib = None


def lib_path() -> str:
    return _LIB_PATH


PIPE_KINDS = {"fp64_mul_add": 0, "fp64_fma": 1, "fp32_mul_add": 2, "fp32_fma": 3}


def pipe_peak(kind: str) -> float:
    """Measured arithmetic operations per second of one pipe mix on the current device
    (se2gpu_pipe_peak; a fused multiply-add counts two)."""
    out = C.c_double(0.0)
    rc = lib().se2gpu_pipe_peak(PIPE_KINDS[kind], C.byref(out))
    if rc != 0:
        raise GpuError(f"se2gpu_pipe_peak failed ({rc}): {lib().se2gpu_last_error(None).decode()}")
    return out.value


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise RuntimeError(f"{_LIB_PATH} is missing: the CUDA library must be built (__graft_entry__.build())")
        L = C.CDLL(_LIB_PATH)
        vp = C.c_void_p
        L.se2gpu_create.argtypes = [C.POINTER(_CProblem), C.c_int, C.c_int, C.POINTER(vp)]
        L.se2gpu_destroy.argtypes = [vp]
        L.se2gpu_destroy.restype = None
        L.se2gpu_last_error.argtypes = [vp]
        L.se2gpu_last_error.restype = C.c_char_p
        L.se2gpu_create_error.restype = C.c_char_p
        L.se2gpu_set_stream.argtypes = [vp, vp]
        L.se2gpu_synchronize.argtypes = [vp]
        L.se2gpu_selftest_wait_expiry.argtypes = [vp, _dp]
        L.se2gpu_set_fields.argtypes = [vp, _dp, _dp, _dp]
        L.se2gpu_get_fields.argtypes = [vp, _dp, _dp, _dp]
        L.se2gpu_advance.argtypes = [vp, C.c_int, _dp]
        L.se2gpu_traces.argtypes = [vp, _dp, C.c_int]
        L.se2gpu_norms.argtypes = [vp, _dp]
        L.se2gpu_assemble_linear_form.argtypes = [vp, _dp, _dp]
        L.se2gpu_assemble_linear_form_device.argtypes = [vp, vp, vp]
        L.se2gpu_info.argtypes = [vp, C.POINTER(C.c_long)]
        L.se2gpu_device_fields.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]
        L.se2gpu_tile_configs.argtypes = [vp, _ip, _ip, C.c_int]
        L.se2gpu_tile_config_info.argtypes = [vp, C.c_int, _ip]
        L.se2gpu_set_tile_config.argtypes = [vp, C.c_int]
        L.se2gpu_tile_config.argtypes = [vp]
        L.se2gpu_ensemble_create.argtypes = [C.POINTER(_CProblem), C.c_int, C.c_int, C.c_int, C.POINTER(vp)]
        L.se2gpu_ensemble_destroy.argtypes = [vp]
        L.se2gpu_ensemble_destroy.restype = None
        L.se2gpu_ensemble_last_error.argtypes = [vp]
        L.se2gpu_ensemble_last_error.restype = C.c_char_p
        L.se2gpu_ensemble_set_stream.argtypes = [vp, vp]
        L.se2gpu_ensemble_set_graphs.argtypes = [vp, C.c_int]
        L.se2gpu_ensemble_set_tile_config.argtypes = [vp, C.c_int, C.c_int]
        L.se2gpu_ensemble_tile_config.argtypes = [vp, C.c_int]
        L.se2gpu_ensemble_advance.argtypes = [vp, C.c_int, _dp, _dp]
        L.se2gpu_ensemble_enqueue.argtypes = [vp, C.c_int]
        L.se2gpu_ensemble_synchronize.argtypes = [vp]
        L.se2gpu_ensemble_get_fields.argtypes = [vp, C.c_int, _dp, _dp, _dp]
        L.se2gpu_ensemble_set_fields.argtypes = [vp, C.c_int, _dp, _dp, _dp]
        L.se2gpu_ensemble_info.argtypes = [vp, C.POINTER(C.c_long)]
        L.se2gpu_norms_device_noalloc.argtypes = [vp, vp, C.c_long, vp, _dp]
        L.se2gpu_pipe_peak.argtypes = [C.c_int, _dp]
        L.se2gpu_checkpoint_size.argtypes = [vp]
        L.se2gpu_checkpoint_size.restype = C.c_long
        L.se2gpu_checkpoint_save.argtypes = [vp, vp, C.c_long]
        L.se2gpu_checkpoint_load.argtypes = [vp, vp, C.c_long]
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray], t=_dp):
    return None if a is None else a.ctypes.data_as(t)


class GpuError(RuntimeError):
    pass


def _problem(s: Setup):
    """se2gpu_problem of a host set-up, with the arrays it points into."""
    keep = [np.ascontiguousarray(x) for x in (s.D.reshape(-1), s.wq, s.w1d, s.J00, s.J11, s.iJ00, s.iJ11,
                                              s.lam, s.mu, s.mass, s.src_elem, s.src_vals.reshape(-1),
                                              s.rec_node, s.rec_elem, s.rec_gll)]
    (D, wq, w1d, J00, J11, iJ00, iJ11, lam, mu, mass, se, sv, rn, re, rg) = keep
    pr = _CProblem(mx=s.mx, my=s.my, p=s.p, dt=s.dt, D=_p(D), wq=_p(wq), w1d=_p(w1d), J00=_p(J00), J11=_p(J11),
                   iJ00=_p(iJ00), iJ11=_p(iJ11), lambda_=_p(lam), mu=_p(mu), mass=_p(mass),
                   nsrc=s.nsrc, src_elem=_p(se, _ip), src_vals=_p(sv),
                   nrec=s.nrec, rec_node=_p(rn, _ip), rec_elem=_p(re, _ip), rec_gll=_p(rg, _ip))
    return pr, keep


class Solver:
    """One problem resident on the GPU, advanced by the fused sm_103a step kernel.

    Mirrors the reference driver: ``advance`` runs the body of the time loop of
    se2wave.c:4722-4775 for n steps, evaluating the source-time functions on the
    host per step as the reference does; ``traces`` returns the per-step
    receiver rows of RecordUVA_MultipleStations_NearestGLL (time first).
    """

    def __init__(self, setup: Setup, precision="fp64", trace_capacity: Optional[int] = None):
        self.setup = setup
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        pr, self._keep = _problem(setup)
        s = setup
        if trace_capacity is None:
            trace_capacity = max(1, min(s.nsteps, 1 << 16)) if s.nrec else 0
        self.trace_capacity = int(trace_capacity)
        h = C.c_void_p()
        rc = lib().se2gpu_create(C.byref(pr), self.precision, self.trace_capacity, C.byref(h))
        if rc != 0:
            raise GpuError(f"se2gpu_create failed ({rc}): {lib().se2gpu_create_error().decode()}")
        self._h = h
        self.tile_config = self._check(lib().se2gpu_tile_config(h), "se2gpu_tile_config")
        self.time = 0.0
        self.step = 0
        self._times = []

    def _check(self, rc: int, what: str) -> int:
        if rc < 0:
            raise GpuError(f"{what} failed ({rc}): {lib().se2gpu_last_error(self._h).decode()}")
        return rc

    def close(self):
        if getattr(self, "_h", None):
            lib().se2gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int):
        self._check(lib().se2gpu_set_stream(self._h, C.c_void_p(stream_ptr)), "se2gpu_set_stream")

    def synchronize(self):
        self._check(lib().se2gpu_synchronize(self._h), "se2gpu_synchronize")

    def advance(self, nsteps: int, stf: Optional[np.ndarray] = None):
        """Advance nsteps (the host evaluates the STFs unless `stf` is given)."""
        if nsteps <= 0:
            return
        times, stf_auto, t_end = self.setup.stf_block(self.time, nsteps)
        if stf is None:
            stf = stf_auto
        stf = np.ascontiguousarray(stf, dtype=np.float64).reshape(-1)
        self._check(lib().se2gpu_advance(self._h, nsteps, _p(stf) if stf.size else None), "se2gpu_advance")
        if self.setup.nrec:
            self._times.extend(times.tolist())
        self.time = t_end
        self.step += nsteps

    def run(self, nsteps: Optional[int] = None, block: int = 1000) -> np.ndarray:
        """Advance to the end of the reference's loop (or nsteps) and return the traces."""
        n = self.setup.nsteps - self.step if nsteps is None else nsteps
        rows = []
        while n > 0:
            k = min(n, block, self.trace_capacity) if self.setup.nrec else min(n, block)
            self.advance(k)
            n -= k
            if self.setup.nrec:
                rows.append(self.traces())
        if not rows:
            return np.zeros((0, 1 + 7 * self.setup.nrec))
        return np.concatenate(rows, axis=0)

    def traces(self) -> np.ndarray:
        """Buffered receiver rows [time, (ux uy vx vy ax ay curl) per receiver], oldest first."""
        nrec = self.setup.nrec
        cap = max(self.trace_capacity, 1)
        out = np.zeros((cap, 7 * max(nrec, 1)))
        n = self._check(lib().se2gpu_traces(self._h, _p(out), cap), "se2gpu_traces")
        times = np.array(self._times[:n])
        del self._times[:n]
        return np.concatenate([times.reshape(-1, 1), out[:n, : 7 * nrec]], axis=1)

    def fields(self):
        n = self.setup.ndof
        u, v, a = np.zeros(n), np.zeros(n), np.zeros(n)
        self._check(lib().se2gpu_get_fields(self._h, _p(u), _p(v), _p(a)), "se2gpu_get_fields")
        return u, v, a

    def set_fields(self, u=None, v=None, a=None):
        arrs = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, a)]
        self._check(lib().se2gpu_set_fields(self._h, *[_p(x) for x in arrs]), "se2gpu_set_fields")

    def selftest_wait_expiry(self):
        """Run the step kernels' bounded wait on a barrier nothing arrives at.  Returns
        (status, seconds the wait took, message); the handle is failed afterwards."""
        sec = C.c_double(0.0)
        rc = lib().se2gpu_selftest_wait_expiry(self._h, C.byref(sec))
        return rc, sec.value, lib().se2gpu_last_error(self._h).decode()

    def norms(self) -> np.ndarray:
        out = np.zeros(6)
        self._check(lib().se2gpu_norms(self._h, _p(out)), "se2gpu_norms")
        return out

    def assemble_linear_form(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        F = np.zeros(self.setup.ndof)
        self._check(lib().se2gpu_assemble_linear_form(self._h, _p(u), _p(F)), "se2gpu_assemble_linear_form")
        return F

    def assemble_linear_form_device(self, u_ptr: int, F_ptr: int):
        self._check(lib().se2gpu_assemble_linear_form_device(self._h, C.c_void_p(u_ptr), C.c_void_p(F_ptr)),
                    "se2gpu_assemble_linear_form_device")

    def info(self) -> dict:
        a = (C.c_long * 9)()
        self._check(lib().se2gpu_info(self._h, a), "se2gpu_info")
        keys = ["nx_g", "ny_g", "p", "precision", "nsrc", "nrec", "launches", "rows", "pitch"]
        return dict(zip(keys, list(a)))

    def device_fields(self):
        u, v, a = C.c_void_p(), C.c_void_p(), C.c_void_p()
        self._check(lib().se2gpu_device_fields(self._h, C.byref(u), C.byref(v), C.byref(a)), "se2gpu_device_fields")
        return u.value, v.value, a.value

    def tile_configs(self):
        """[(elements per tile edge, threads per CTA)] the step kernel offers for this problem."""
        e = np.zeros(16, dtype=np.int32)
        t = np.zeros(16, dtype=np.int32)
        n = self._check(lib().se2gpu_tile_configs(self._h, _p(e, _ip), _p(t, _ip), 16), "se2gpu_tile_configs")
        return [(int(e[i]), int(t[i])) for i in range(n)]

    def tile_config_info(self, config: int) -> dict:
        """One configuration in full (se2gpu_tile_config_info)."""
        info = np.zeros(4, dtype=np.int32)
        self._check(lib().se2gpu_tile_config_info(self._h, int(config), _p(info, _ip)), "se2gpu_tile_config_info")
        return {"edge": int(info[0]), "threads": int(info[1]), "owned_buffers": int(info[2]),
                "ctas_per_sm": int(info[3])}

    def set_tile_config(self, config: int):
        self._check(lib().se2gpu_set_tile_config(self._h, int(config)), "se2gpu_set_tile_config")
        self.tile_config = int(config)

    def checkpoint(self) -> bytes:
        """The handle's state (se2gpu_checkpoint_save; buffered trace rows must have been fetched),
        followed by this binding's time, step count and the times of rows still pending."""
        n = self._check(lib().se2gpu_checkpoint_size(self._h), "se2gpu_checkpoint_size")
        buf = C.create_string_buffer(n)
        self._check(lib().se2gpu_checkpoint_save(self._h, buf, n), "se2gpu_checkpoint_save")
        pend = np.array(self._times, dtype=np.float64)
        return buf.raw + pend.tobytes() + np.array([self.time, self.step, len(pend)], dtype=np.float64).tobytes()

    def restore(self, blob: bytes):
        time_, step, npend = np.frombuffer(blob[-24:], dtype=np.float64)
        npend = int(npend)
        body = blob[:len(blob) - 24 - 8 * npend]
        self._check(lib().se2gpu_checkpoint_load(self._h, body, len(body)), "se2gpu_checkpoint_load")
        self.time, self.step = float(time_), int(step)
        self._times = np.frombuffer(blob[len(body):len(blob) - 24], dtype=np.float64).tolist()


class Ensemble:
    """Many independent shots advanced together by the batched persistent kernel
    (se2gpu_ensemble_*): one launch per degree group per step, blocks of
    `block` steps replayed as CUDA graphs.  FP32 precisions only; each shot
    evolves bit-identically to a :class:`Solver` of the same set-up."""

    def __init__(self, setups, precision="fp32_kahan", block: int = 100):
        self.setups = list(setups)
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        n = len(self.setups)
        arr = (_CProblem * n)()
        self._keep = []
        for i, su in enumerate(self.setups):
            pr, keep = _problem(su)
            arr[i] = pr
            self._keep.append(keep)
        h = C.c_void_p()
        rc = lib().se2gpu_ensemble_create(arr, n, self.precision, int(block), C.byref(h))
        self._keep = None   # the library copied everything it needs
        if rc != 0:
            raise GpuError(f"se2gpu_ensemble_create failed ({rc}): {lib().se2gpu_ensemble_last_error(None).decode()}")
        self._h = h
        self.block = int(block)
        self.nsrc = np.array([su.nsrc for su in self.setups])
        self.nrec = np.array([su.nrec for su in self.setups])
        self.time = np.zeros(n)
        self.step = 0

    def _check(self, rc: int, what: str) -> int:
        if rc < 0:
            raise GpuError(f"{what} failed ({rc}): {lib().se2gpu_ensemble_last_error(self._h).decode()}")
        return rc

    def close(self):
        if getattr(self, "_h", None):
            lib().se2gpu_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __len__(self):
        return len(self.setups)

    def stf(self, nsteps: int):
        """Host STF values of the next nsteps steps, shot-major, and each shot's times."""
        vals, times, ends = [], [], []
        for i, su in enumerate(self.setups):
            t, v, t_end = su.stf_block(self.time[i], nsteps)
            vals.append(v.reshape(-1))
            times.append(t)
            ends.append(t_end)
        return np.ascontiguousarray(np.concatenate(vals) if vals else np.zeros(0)), times, np.array(ends)

    def advance(self, nsteps: int, stf: Optional[np.ndarray] = None, traces: bool = True):
        """Advance every shot; returns per shot the receiver rows [time, 7 per receiver] (or None)."""
        if nsteps <= 0:
            return [np.zeros((0, 1 + 7 * r)) for r in self.nrec] if traces else None
        auto, times, ends = self.stf(nsteps)
        stf = auto if stf is None else np.ascontiguousarray(stf, dtype=np.float64).reshape(-1)
        out = np.zeros(max(1, nsteps * 7 * int(self.nrec.sum()))) if traces else None
        self._check(lib().se2gpu_ensemble_advance(self._h, int(nsteps), _p(stf) if stf.size else None, _p(out)),
                    "se2gpu_ensemble_advance")
        self.time = ends
        self.step += nsteps
        if not traces:
            return None
        res, off = [], 0
        for i, r in enumerate(self.nrec):
            blk = out[off: off + nsteps * 7 * r].reshape(nsteps, 7 * r)
            res.append(np.concatenate([times[i].reshape(-1, 1), blk], axis=1))
            off += nsteps * 7 * r
        return res

    def enqueue(self, nsteps: int):
        self._check(lib().se2gpu_ensemble_enqueue(self._h, int(nsteps)), "se2gpu_ensemble_enqueue")
        self.step += nsteps

    def synchronize(self):
        self._check(lib().se2gpu_ensemble_synchronize(self._h), "se2gpu_ensemble_synchronize")

    def set_stream(self, stream_ptr: int):
        self._check(lib().se2gpu_ensemble_set_stream(self._h, C.c_void_p(stream_ptr)), "se2gpu_ensemble_set_stream")

    def set_graphs(self, enable: bool):
        self._check(lib().se2gpu_ensemble_set_graphs(self._h, int(bool(enable))), "se2gpu_ensemble_set_graphs")

    def set_tile_config(self, p: int, config: int):
        self._check(lib().se2gpu_ensemble_set_tile_config(self._h, int(p), int(config)),
                    "se2gpu_ensemble_set_tile_config")

    def tile_config(self, p: int) -> int:
        return self._check(lib().se2gpu_ensemble_tile_config(self._h, int(p)), "se2gpu_ensemble_tile_config")

    def degrees(self):
        return sorted({su.p for su in self.setups})

    def fields(self, shot: int):
        if not 0 <= shot < len(self.setups):   # let the library report the bad index
            self._check(lib().se2gpu_ensemble_get_fields(self._h, int(shot), None, None, None),
                        "se2gpu_ensemble_get_fields")
        n = self.setups[shot].ndof
        u, v, a = np.zeros(n), np.zeros(n), np.zeros(n)
        self._check(lib().se2gpu_ensemble_get_fields(self._h, int(shot), _p(u), _p(v), _p(a)),
                    "se2gpu_ensemble_get_fields")
        return u, v, a

    def set_fields(self, shot: int, u=None, v=None, a=None):
        arrs = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, a)]
        self._check(lib().se2gpu_ensemble_set_fields(self._h, int(shot), *[_p(x) for x in arrs]),
                    "se2gpu_ensemble_set_fields")

    def info(self) -> dict:
        a = (C.c_long * 9)()
        self._check(lib().se2gpu_ensemble_info(self._h, a), "se2gpu_ensemble_info")
        keys = ["shots", "groups", "block", "launches", "replays", "nodes", "sources", "receivers", "items"]
        return dict(zip(keys, list(a)))
