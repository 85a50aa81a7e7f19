"""ctypes wrapper of the oracle port (oracle/se2_oracle.c) and of the reference
driver built in place (oracle/_ref/ref_driver).

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the CPU
baseline legs of bench.py use this module, and only as the values results are
compared with or as the timed CPU implementation; the product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libse2oracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _CSpec(C.Structure):
    _fields_ = [("mx", C.c_int), ("my", C.c_int), ("p", C.c_int),
                ("scale", C.c_double * 2), ("shift", C.c_double * 2),
                ("cell_vp", _dp), ("cell_vs", _dp), ("cell_rho", _dp),
                ("vp", C.c_double), ("vs", C.c_double), ("rho", C.c_double),
                ("cfl", C.c_double), ("dt", C.c_double), ("tmax", C.c_double),
                ("nt", C.c_int), ("nearest_internal_gll", C.c_int),
                ("nsrc", C.c_int), ("src_xy", _dp), ("src_m", _dp), ("stf_type", _ip), ("stf_par", _dp),
                ("nrec", C.c_int), ("rec_xy", _dp),
                ("perturb", C.c_int), ("dvp", C.c_double), ("dvs", C.c_double), ("drho", C.c_double)]


def build(quiet: bool = True) -> str:
    """Compile the oracle port (and nothing else)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.se2o_create.argtypes = [C.POINTER(_CSpec), C.POINTER(C.c_void_p)]
        L.se2o_create.restype = C.c_int
        L.se2o_destroy.argtypes = [C.c_void_p]
        L.se2o_last_error.restype = C.c_char_p
        L.se2o_info.argtypes = [C.c_void_p, _ip, _dp]
        L.se2o_get.argtypes = [C.c_void_p, C.c_char_p, _dp, C.c_long]
        L.se2o_run.argtypes = [C.c_void_p, C.c_long, _dp, _dp, C.c_long]
        L.se2o_run.restype = C.c_long
        L.se2o_get_state.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.se2o_set_state.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_double]
        L.se2o_force.argtypes = [C.c_void_p, _dp, _dp]
        L.se2o_stf.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_long, _dp]
        L.se2o_bench.argtypes = [C.POINTER(_CSpec), C.c_int, C.c_long, C.c_long, C.c_int]
        L.se2o_bench.restype = C.c_double
        _lib = L
    return _lib


def _ptr(a: Optional[np.ndarray], t=_dp):
    return None if a is None else a.ctypes.data_as(t)


class _SpecHolder:
    """Keeps the numpy buffers alive while the C struct points at them."""

    def __init__(self, spec):
        self.keep = []
        cs = _CSpec()
        cs.mx, cs.my, cs.p = spec.mx, spec.my, spec.p
        cs.scale[0], cs.scale[1] = spec.scale
        cs.shift[0], cs.shift[1] = spec.shift
        cells = spec.cell_arrays()
        if cells is not None:
            self.keep += list(cells)
            cs.cell_vp, cs.cell_vs, cs.cell_rho = (_ptr(c) for c in cells)
        cs.vp, cs.vs, cs.rho = spec.vp, spec.vs, spec.rho
        cs.cfl, cs.dt, cs.tmax, cs.nt = spec.cfl, spec.dt, spec.tmax, spec.nt
        cs.nearest_internal_gll = int(spec.nearest_internal_gll)
        ns = len(spec.sources)
        sxy = np.array([[s.x, s.y] for s in spec.sources], dtype=np.float64).reshape(-1)
        sm = np.array([list(s.moment) for s in spec.sources], dtype=np.float64).reshape(-1)
        st = np.array([s.stf for s in spec.sources], dtype=np.int32).reshape(-1)
        sp = np.array([list(s.par) for s in spec.sources], dtype=np.float64).reshape(-1)
        rxy = np.array(spec.receivers, dtype=np.float64).reshape(-1)
        self.keep += [sxy, sm, st, sp, rxy]
        cs.nsrc = ns
        cs.src_xy, cs.src_m, cs.stf_type, cs.stf_par = _ptr(sxy), _ptr(sm), _ptr(st, _ip), _ptr(sp)
        cs.nrec = len(spec.receivers)
        cs.rec_xy = _ptr(rxy)
        if spec.perturb is not None:
            cs.perturb = 1
            cs.dvp, cs.dvs, cs.drho = spec.perturb
        self.cs = cs


class OracleSolver:
    """The reference algorithm on the CPU (see oracle/se2_oracle.c)."""

    def __init__(self, spec):
        self.spec = spec
        self._h = _SpecHolder(spec)
        self._ctx = C.c_void_p()
        if lib().se2o_create(C.byref(self._h.cs), C.byref(self._ctx)) != 0:
            raise RuntimeError("oracle set-up failed: " + lib().se2o_last_error().decode())
        ints = (C.c_int * 6)()
        dbls = (C.c_double * 3)()
        lib().se2o_info(self._ctx, ints, dbls)
        self.nx_g, self.ny_g, self.n1, self.nsteps_planned, self.nrec, self.nsrc = list(ints)
        self.dt, self.dt_cfl, self.tmax = list(dbls)
        self.ndof = 2 * self.nx_g * self.ny_g

    def __del__(self):
        if getattr(self, "_ctx", None):
            lib().se2o_destroy(self._ctx)
            self._ctx = None

    def get(self, name: str) -> np.ndarray:
        sizes = {"xi": self.n1, "w1d": self.n1, "w": self.n1 ** 2, "D": self.n1 ** 2,
                 "dN_dxi": self.n1 ** 4, "dN_deta": self.n1 ** 4, "coords": self.ndof, "mass": self.ndof,
                 "cell_lmr": 3 * self.spec.ne, "src_values": self.nsrc * 2 * self.n1 ** 2,
                 "src_index": 2 * self.nsrc, "rec_index": 3 * self.nrec}
        out = np.zeros(max(sizes[name], 1), dtype=np.float64)
        if lib().se2o_get(self._ctx, name.encode(), _ptr(out), out.size) != 0:
            raise RuntimeError(lib().se2o_last_error().decode())
        return out[:sizes[name]]

    def run(self, nsteps: int, traces: bool = True, norms: bool = False):
        width = 1 + 7 * self.nrec
        tr = np.zeros((max(nsteps, 1), width), dtype=np.float64) if traces else None
        nr = np.zeros((nsteps // 100 + 1, 7), dtype=np.float64) if norms else None
        n = lib().se2o_run(self._ctx, nsteps, _ptr(tr), _ptr(nr), 0 if nr is None else nr.shape[0])
        if n < 0:
            raise RuntimeError(lib().se2o_last_error().decode())
        res = {"nsteps": int(n)}
        if tr is not None:
            res["traces"] = tr[:n]
        if nr is not None:
            res["norms"] = nr[: int((nr[:, 0] > 0).sum())]
        return res

    def state(self):
        u, v, a = (np.zeros(self.ndof) for _ in range(3))
        lib().se2o_get_state(self._ctx, _ptr(u), _ptr(v), _ptr(a))
        return u, v, a

    def set_state(self, u, v, a, time=0.0):
        u, v, a = (np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, a))
        lib().se2o_set_state(self._ctx, _ptr(u), _ptr(v), _ptr(a), float(time))

    def force(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        F = np.zeros(self.ndof)
        lib().se2o_force(self._ctx, _ptr(u), _ptr(F))
        return F


def stf(type_: int, par, t0: float, dt: float, n: int) -> np.ndarray:
    par = np.ascontiguousarray(par, dtype=np.float64)
    out = np.zeros(n)
    if lib().se2o_stf(type_, _ptr(par), t0, dt, n, _ptr(out)) != 0:
        raise RuntimeError(lib().se2o_last_error().decode())
    return out


def bench(spec, nthreads: int, warmup: int, nsteps: int, record: bool = True) -> float:
    """Wall seconds for nsteps of nthreads independent oracle solves (max over threads)."""
    h = _SpecHolder(spec)
    t = lib().se2o_bench(C.byref(h.cs), nthreads, warmup, nsteps, int(record))
    if t < 0:
        raise RuntimeError("oracle bench failed: " + lib().se2o_last_error().decode())
    return t


# ---------------------------------------------------------------------------
# the reference itself, compiled in place (only where the reference tree exists)
# ---------------------------------------------------------------------------
def build_ref(refdir: Optional[str] = None) -> bool:
    """Compile the reference in place (oracle/Makefile target ref-if-present) from refdir,
    else from the SE2_REFERENCE_DIR environment variable, else from the recipe's default
    tree.  Returns whether the driver exists afterwards."""
    extra = [f"REFDIR={refdir}"] if refdir else []
    subprocess.run(["make", "-s", "-C", HERE, "ref-if-present", *extra], check=True, stdout=subprocess.DEVNULL)
    return os.path.exists(REF_DRIVER)


def ref_source_vector(spec, impl: int, extra_args=()) -> np.ndarray:
    """The reference's assembled source vector of spec's first source by implementation
    impl (0 pointwise, 2 cubic-spline kernel, 3 P0); extra_args e.g. ["-sm_h", "40"]."""
    with tempfile.TemporaryDirectory() as d:
        sfile = os.path.join(d, "spec.txt")
        cells = spec.cell_arrays()
        cell_file = None
        if cells is not None:
            cell_file = os.path.join(d, "cells.bin")
            np.concatenate(cells).astype(np.float64).tofile(cell_file)
        with open(sfile, "w") as f:
            f.write(spec.to_text(cell_file))
        r = subprocess.run([REF_DRIVER, "srcvec", sfile, str(impl), d, *extra_args], cwd=d, capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-2000:] + r.stdout[-2000:])
        return np.fromfile(os.path.join(d, "g.bin"), dtype=np.float64)


def ref_run(spec, extra_args=(), force_u: Optional[np.ndarray] = None) -> dict:
    """Run the reference's own code on `spec`; return its binary dumps."""
    with tempfile.TemporaryDirectory() as d:
        cell_file = None
        cells = spec.cell_arrays()
        if cells is not None:
            cell_file = os.path.join(d, "cells.bin")
            np.concatenate(cells).astype(np.float64).tofile(cell_file)
        sfile = os.path.join(d, "spec.txt")
        with open(sfile, "w") as f:
            f.write(spec.to_text(cell_file))
        out = {}
        if force_u is not None:
            ufile = os.path.join(d, "u_in.bin")
            np.ascontiguousarray(force_u, dtype=np.float64).tofile(ufile)
            r = subprocess.run([REF_DRIVER, "force", sfile, ufile, d, *extra_args], cwd=d, capture_output=True, text=True)
        else:
            r = subprocess.run([REF_DRIVER, "run", sfile, d, *extra_args], cwd=d, capture_output=True, text=True)
        out["stdout"], out["stderr"], out["returncode"] = r.stdout, r.stderr, r.returncode
        if r.returncode != 0:
            return out
        for fn in os.listdir(d):
            path = os.path.join(d, fn)
            if fn.endswith(".bin") and fn not in ("cells.bin", "u_in.bin"):
                dt = np.int32 if fn == "src_index.bin" else np.float64
                out[fn[:-4]] = np.fromfile(path, dtype=dt)
            elif fn.endswith(".dat") or fn.endswith(".mpimeta") or fn == "norms.txt":
                with open(path) as fh:
                    out[fn] = fh.read()
        if "trace_capture" in out:
            width = 1 + 7 * len(spec.receivers)
            out["traces"] = out["trace_capture"].reshape(-1, width)
        if "interp_capture" in out:   # RecordUV_interp rows: time ux uy vx vy
            out["interp"] = out["interp_capture"].reshape(-1, 5)
            for line in r.stdout.splitlines():   # its first call prints the interpolated coordinate
                if "interpolated coordinate" in line:
                    out["interp_xri_text"] = np.array([float(t) for t in line.split("-->")[1].split()])
        return out


def ref_stf(kind: str, a: float, b: float, c: float, t0: float, dt: float, n: int) -> np.ndarray:
    with tempfile.TemporaryDirectory() as d:
        fn = os.path.join(d, "stf.bin")
        subprocess.run([REF_DRIVER, "stf", kind, repr(a), repr(b), repr(c), repr(t0), repr(dt), str(n), fn], check=True,
                       capture_output=True)
        return np.fromfile(fn, dtype=np.float64).reshape(n, 2)
