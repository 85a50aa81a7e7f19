"""ctypes binding of the FP64 host set-up library (include/se2host.h, lib/libse2host.so).

The set-up runs in C, as the reference's does; Python only marshals arrays.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Tuple

import numpy as np

from .spec import Spec

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libse2host.so")
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
                ("perturb", C.c_int), ("dvp", C.c_double), ("dvs", C.c_double), ("drho", C.c_double),
                ("src_impl", C.c_int), ("sm_h", C.c_double),
                ("ninterp", C.c_int), ("interp_xy", _dp)]


class _CSetup(C.Structure):
    _fields_ = [("mx", C.c_int), ("my", C.c_int), ("p", C.c_int), ("n1", C.c_int), ("npe", C.c_int),
                ("nx_g", C.c_int), ("ny_g", C.c_int), ("nnodes", C.c_long),
                ("xi", _dp), ("w1d", _dp), ("wq", _dp), ("D", _dp), ("xnode", _dp), ("ynode", _dp),
                ("J00", _dp), ("J11", _dp), ("iJ00", _dp), ("iJ11", _dp),
                ("lambda_", _dp), ("mu", _dp), ("rho", _dp), ("mass", _dp),
                ("gmin", C.c_double * 2), ("gmax", C.c_double * 2),
                ("dt_cfl", C.c_double), ("dt", C.c_double), ("tmax", C.c_double),
                ("nt", C.c_long), ("nsteps", C.c_long),
                ("nsrc", C.c_int), ("src_elem", _ip), ("src_gll", _ip), ("src_vals", _dp),
                ("stf_type", _ip), ("stf_par", _dp),
                ("nrec", C.c_int), ("rec_xy", _dp), ("rec_node", _ip), ("rec_elem", _ip), ("rec_gll", _ip),
                ("nsrc_phys", C.c_int), ("src_owner", _ip),
                ("nrec_sta", C.c_int), ("ninterp", C.c_int), ("interp_xy", _dp), ("interp_elem", _ip),
                ("interp_N", _dp), ("interp_xri", _dp)]


class CShotDraw(C.Structure):
    _fields_ = [("mx", C.c_int), ("my", C.c_int), ("p", C.c_int), ("nrec", C.c_int), ("nsteps", C.c_long),
                ("h", C.c_double), ("Lx", C.c_double), ("Ly", C.c_double), ("interface_y", C.c_double),
                ("lower", C.c_double * 3), ("upper", C.c_double * 3), ("ninc", C.c_int),
                ("inc", (C.c_double * 8) * 2), ("src_xy", C.c_double * 2), ("moment", C.c_double * 4),
                ("f0", C.c_double), ("t0", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise RuntimeError(f"{_LIB_PATH} is missing: run __graft_entry__.build() (or se2dr_fork_gb300.build)")
        L = C.CDLL(_LIB_PATH)
        L.se2_host_last_error.restype = C.c_char_p
        L.se2_setup_create.argtypes = [C.POINTER(_CSpec), C.POINTER(C.POINTER(_CSetup))]
        L.se2_setup_destroy.argtypes = [C.POINTER(_CSetup)]
        L.se2_gll.argtypes = [C.c_int, _dp, _dp]
        L.se2_basis_1d.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.se2_basis_deriv_1d.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.se2_stf_block.argtypes = [C.POINTER(_CSetup), _dp, C.c_long, _dp, _dp]
        L.se2_stf_eval.argtypes = [C.c_int, _dp, C.c_double, _dp]
        L.se2_gaussian_random_field.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                                C.c_ulonglong, _dp]
        L.se2_source_vector.argtypes = [C.POINTER(_CSetup), C.c_int, C.c_double, _dp, _dp, _dp]
        L.se2_interp_receiver.argtypes = [C.POINTER(_CSetup), _dp, _ip, _dp, _dp]
        L.se2_interp_rows.argtypes = [C.POINTER(_CSetup), C.c_long, _dp, _dp]
        L.se2_shot_draw_params.argtypes = [C.c_ulonglong, C.c_long, C.c_int, C.POINTER(CShotDraw)]
        L.se2_shot_materials.argtypes = [C.POINTER(CShotDraw), _dp, _dp, _dp]
        L.se2_write_vts.argtypes = [C.POINTER(_CSetup), C.c_char_p, C.c_int, C.POINTER(C.c_char_p),
                                    C.POINTER(_dp)]
        _lib = L
    return _lib


def _err() -> str:
    return lib().se2_host_last_error().decode()


def _p(a: Optional[np.ndarray], t=_dp):
    return None if a is None else a.ctypes.data_as(t)


class _SpecHolder:
    def __init__(self, spec: Spec):
        self.keep = []
        cs = _CSpec()
        cs.mx, cs.my, cs.p = spec.mx, spec.my, spec.p
        cs.scale[0], cs.scale[1] = spec.scale
        cs.shift[0], cs.shift[1] = spec.shift
        cells = spec.cell_arrays()
        if cells is not None:
            self.keep += list(cells)
            cs.cell_vp, cs.cell_vs, cs.cell_rho = (_p(c) for c in cells)
        cs.vp, cs.vs, cs.rho = spec.vp, spec.vs, spec.rho
        cs.cfl, cs.dt, cs.tmax, cs.nt = spec.cfl, spec.dt, spec.tmax, spec.nt
        cs.nearest_internal_gll = int(spec.nearest_internal_gll)
        sxy = np.array([[s.x, s.y] for s in spec.sources], dtype=np.float64).reshape(-1)
        sm = np.array([list(s.moment) for s in spec.sources], dtype=np.float64).reshape(-1)
        st = np.array([s.stf for s in spec.sources], dtype=np.int32).reshape(-1)
        sp = np.array([list(s.par) for s in spec.sources], dtype=np.float64).reshape(-1)
        rxy = np.array(spec.receivers, dtype=np.float64).reshape(-1)
        self.keep += [sxy, sm, st, sp, rxy]
        cs.nsrc = len(spec.sources)
        cs.src_xy, cs.src_m, cs.stf_type, cs.stf_par = _p(sxy), _p(sm), _p(st, _ip), _p(sp)
        cs.nrec = len(spec.receivers)
        cs.rec_xy = _p(rxy)
        if spec.perturb is not None:
            cs.perturb = 1
            cs.dvp, cs.dvs, cs.drho = spec.perturb
        cs.src_impl, cs.sm_h = int(spec.src_impl), float(spec.sm_h)
        ixy = np.array(spec.interp_receivers, dtype=np.float64).reshape(-1)
        self.keep.append(ixy)
        cs.ninterp = len(spec.interp_receivers)
        cs.interp_xy = _p(ixy)
        self.cs = cs


def _arr(ptr, n, dtype=np.float64) -> np.ndarray:
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class Setup:
    """FP64 host set-up of a :class:`Spec` (se2_setup_create)."""

    def __init__(self, spec: Spec):
        self.spec = spec
        h = _SpecHolder(spec)
        ptr = C.POINTER(_CSetup)()
        if lib().se2_setup_create(C.byref(h.cs), C.byref(ptr)) != 0:
            raise ValueError("set-up failed: " + _err())
        self._ptr = ptr
        s = ptr.contents
        self.mx, self.my, self.p, self.n1, self.npe = s.mx, s.my, s.p, s.n1, s.npe
        self.nx_g, self.ny_g, self.nnodes = s.nx_g, s.ny_g, int(s.nnodes)
        self.dt, self.dt_cfl, self.tmax = s.dt, s.dt_cfl, s.tmax
        self.nt, self.nsteps = int(s.nt), int(s.nsteps)
        self.nsrc, self.nrec = s.nsrc, s.nrec
        self.gmin, self.gmax = tuple(s.gmin), tuple(s.gmax)
        n1, npe = self.n1, self.npe
        self.xi = _arr(s.xi, n1)
        self.w1d = _arr(s.w1d, n1)
        self.wq = _arr(s.wq, npe)
        self.D = _arr(s.D, npe).reshape(n1, n1)
        self.xnode = _arr(s.xnode, self.nx_g)
        self.ynode = _arr(s.ynode, self.ny_g)
        self.J00, self.iJ00 = _arr(s.J00, self.mx), _arr(s.iJ00, self.mx)
        self.J11, self.iJ11 = _arr(s.J11, self.my), _arr(s.iJ11, self.my)
        ne = self.mx * self.my
        self.lam, self.mu, self.rho = _arr(s.lambda_, ne), _arr(s.mu, ne), _arr(s.rho, ne)
        self.mass = _arr(s.mass, self.nnodes)
        self.src_elem = _arr(s.src_elem, self.nsrc, np.int32)
        self.src_gll = _arr(s.src_gll, self.nsrc, np.int32)
        self.src_vals = _arr(s.src_vals, self.nsrc * 2 * npe).reshape(self.nsrc, 2 * npe)
        self.rec_node = _arr(s.rec_node, self.nrec, np.int32)
        self.rec_elem = _arr(s.rec_elem, self.nrec, np.int32)
        self.rec_gll = _arr(s.rec_gll, self.nrec, np.int32)
        self.nsrc_phys = s.nsrc_phys
        self.src_owner = _arr(s.src_owner, self.nsrc, np.int32)
        # receiver list = nrec_sta stations, then npe element nodes per interpolating receiver
        self.nrec_sta, self.ninterp = s.nrec_sta, s.ninterp
        self.interp_elem = _arr(s.interp_elem, self.ninterp, np.int32)
        self.interp_N = _arr(s.interp_N, self.ninterp * npe).reshape(self.ninterp, npe)
        self.interp_xri = _arr(s.interp_xri, 2 * self.ninterp).reshape(self.ninterp, 2)

    def __del__(self):
        if getattr(self, "_ptr", None):
            lib().se2_setup_destroy(self._ptr)
            self._ptr = None

    @property
    def ndof(self) -> int:
        return 2 * self.nnodes

    def coords(self) -> np.ndarray:
        """Interleaved node coordinates, the reference's coordinate Vec layout."""
        X, Y = np.meshgrid(self.xnode, self.ynode)
        return np.stack([X.ravel(), Y.ravel()], axis=1).ravel()

    def mass_vec(self) -> np.ndarray:
        """Lumped mass as the reference's interleaved 2-component Vec (Md)."""
        return np.repeat(self.mass, 2)

    def source_vector(self, impl: int, xy, moment, kernel_h: float = 0.0) -> np.ndarray:
        """Assembled source vector of one moment source (se2_source_vector): impl 0 pointwise,
        2 cubic-spline kernel (radius kernel_h, <= 0 for the reference's default), 3 P0."""
        g = np.zeros(self.ndof)
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        m = np.ascontiguousarray(moment, dtype=np.float64)
        if lib().se2_source_vector(self._ptr, int(impl), float(kernel_h), _p(xy), _p(m), _p(g)) != 0:
            raise ValueError(_err())
        return g

    def interp_receiver(self, xy) -> Tuple[int, np.ndarray, np.ndarray]:
        """(element, weights N[npe], interpolated coordinate) of a point (se2_interp_receiver)."""
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        eid, N, xri = C.c_int(), np.zeros(self.npe), np.zeros(2)
        if lib().se2_interp_receiver(self._ptr, _p(xy), C.byref(eid), _p(N), _p(xri)) != 0:
            raise ValueError(_err())
        return eid.value, N, xri

    def interp_rows(self, rows: np.ndarray) -> np.ndarray:
        """Receiver rows [nsteps][(1 +) 7*nrec] (with or without the time column) -> the
        interpolating receivers' rows [nsteps][ninterp][7] (se2_interp_rows)."""
        rows = np.asarray(rows, dtype=np.float64)
        if rows.shape[1] == 1 + 7 * self.nrec:
            rows = rows[:, 1:]
        rows = np.ascontiguousarray(rows)
        assert rows.shape[1] == 7 * self.nrec
        out = np.zeros((rows.shape[0], self.ninterp, 7))
        if lib().se2_interp_rows(self._ptr, rows.shape[0], _p(rows), _p(out)) != 0:
            raise ValueError(_err())
        return out

    def write_vts(self, path: str, fields: dict):
        """se2_write_vts: a VTK StructuredGrid snapshot over the GLL nodes of nodal fields
        {name: interleaved [node][component] array of 2*nnodes}, arrays <name>_x, <name>_y."""
        names = list(fields)
        arrs = [np.ascontiguousarray(fields[k], dtype=np.float64) for k in names]
        if any(a.size != self.ndof for a in arrs):
            raise ValueError(f"every field needs {self.ndof} values")
        cn = (C.c_char_p * len(names))(*[k.encode() for k in names])
        cv = (_dp * len(arrs))(*[_p(a) for a in arrs])
        if lib().se2_write_vts(self._ptr, str(path).encode(), len(names), cn, cv) != 0:
            raise ValueError(_err())

    def stf_block(self, time: float, n: int) -> Tuple[np.ndarray, np.ndarray, float]:
        """Times and STF values of the next n steps after `time`."""
        t = C.c_double(time)
        times = np.zeros(max(n, 1))
        stf = np.zeros(max(n * self.nsrc, 1))
        if lib().se2_stf_block(self._ptr, C.byref(t), n, _p(times), _p(stf)) != 0:
            raise ValueError(_err())
        return times[:n], stf[: n * self.nsrc].reshape(n, self.nsrc), t.value


def gll(p: int) -> Tuple[np.ndarray, np.ndarray]:
    xi, w = np.zeros(p + 1), np.zeros(p + 1)
    if lib().se2_gll(p, _p(xi), _p(w)) != 0:
        raise ValueError(_err())
    return xi, w


def basis(p: int, x, deriv: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    out = np.zeros((x.size, p + 1))
    fn = lib().se2_basis_deriv_1d if deriv else lib().se2_basis_1d
    if fn(p, x.size, _p(x), _p(out)) != 0:
        raise ValueError(_err())
    return out


def stf_eval(type_: int, par, t: float) -> float:
    par = np.ascontiguousarray(par, dtype=np.float64)
    v = C.c_double()
    if lib().se2_stf_eval(type_, _p(par), t, C.byref(v)) != 0:
        raise ValueError(_err())
    return v.value


def gaussian_random_field(mx: int, my: int, mean: float = 5000.0, rel_std: float = 0.1,
                          corr_cells: float = 8.0, seed: int = 0) -> np.ndarray:
    out = np.zeros(mx * my)
    if lib().se2_gaussian_random_field(mx, my, mean, rel_std, corr_cells, seed, _p(out)) != 0:
        raise ValueError(_err())
    return out


SHOT_ENSEMBLE, SHOT_TRAINING, SHOT_OOD = 0, 1, 2


def shot_draw(seed: int, index: int, kind: int = SHOT_ENSEMBLE) -> CShotDraw:
    """Seeded draw of one shot's mesh, materials, source and wavelet (se2_shot_draw_params)."""
    d = CShotDraw()
    if lib().se2_shot_draw_params(seed, index, kind, C.byref(d)) != 0:
        raise ValueError(_err())
    return d


def shot_materials(d: CShotDraw) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Per-cell (vp, vs, rho) of a drawn shot (2 layers + elliptical inclusions)."""
    n = d.mx * d.my
    vp, vs, rho = np.zeros(n), np.zeros(n), np.zeros(n)
    if lib().se2_shot_materials(C.byref(d), _p(vp), _p(vs), _p(rho)) != 0:
        raise ValueError(_err())
    return vp, vs, rho
