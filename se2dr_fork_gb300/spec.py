"""Problem specifications for the se2wave explicit SEM time loop.

A :class:`Spec` carries everything ``se2wave_demo`` (se2wave.c:4541-4807) hard-codes
or reads from the options database: mesh (``-mx -my -bdegree``), domain scaling
(se2wave.c:4575-4585), cell materials (4592), moment sources with their
source-time functions (4616-4683), receivers (4688-4697), the CFL factor (4709)
and ``-tmax -dt -nt``.

Named workloads:

* :func:`demo` -- the reference demo exactly (se2wave.c:4541-4807).
* :func:`explosion64` -- 64x64 elements, degree 6, 2 km square, homogeneous
  rho=2700, Vp=6000, Vs=3464, explosive source M=diag(1e15,1e15) at the centre,
  Ricker f0=10 Hz t0=0.15 s, dt = 0.2 CFL, tmax 0.4 s, one receiver at (500, 500).
* :func:`grf2048` -- 2048x2048 elements, degree 4, 20 km square, per-cell Vp from a
  seeded Gaussian random field (mean 5000 m/s, 10 % std, correlation length 8
  cells), Vp/Vs = 1.73, rho = 2700, same explosive source with Ricker f0 = 8 Hz,
  t0 = 0.15 s, 64 receivers on a horizontal line, 20000 steps at 0.2 CFL.
* :func:`shot` -- one seeded draw of the ensemble / surrogate distributions:
  2-layer + elliptical-inclusion materials, random source position, symmetric
  moment tensor with N(0, 1e15) entries, Ricker f0 ~ U[5, 20] Hz; receivers on
  the top surface.  :func:`ensemble` is a list of such draws.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

STF_RICKER, STF_GAUSSIAN, STF_YOFFE = 0, 1, 2
_STF_NAMES = {STF_RICKER: "ricker", STF_GAUSSIAN: "gaussian", STF_YOFFE: "yoffe"}


@dataclass
class Source:
    """Moment-tensor point source snapped to the nearest GLL point
    (SOURCE_TYPE_MOMENT, SOURCE_IMPL_NEAREST_QPOINT; se2wave.c:2995-3429)."""
    x: float
    y: float
    moment: Tuple[float, float, float, float]  # [M00, M01, M10, M11]
    stf: int = STF_RICKER
    par: Tuple[float, float, float] = (0.15, 12.0, 1.0)  # Ricker (t0, f0, amp)


@dataclass
class Spec:
    mx: int = 8
    my: int = 8
    p: int = 2
    scale: Tuple[float, float] = (2000.0, 2000.0)
    shift: Tuple[float, float] = (-1000.0, -1000.0)
    vp: float = 4746.3670317412243
    vs: float = 2740.2554625435928
    rho: float = 1000.0
    cell_vp: Optional[np.ndarray] = None
    cell_vs: Optional[np.ndarray] = None
    cell_rho: Optional[np.ndarray] = None
    cfl: float = 0.5
    dt: float = 0.0          # > 0 overrides the CFL step (-dt)
    tmax: float = 0.4        # -tmax
    nt: int = -1             # >= 0 overrides (int)(tmax/dt)+4 (-nt)
    nearest_internal_gll: bool = True
    sources: List[Source] = field(default_factory=list)
    receivers: List[Tuple[float, float]] = field(default_factory=list)
    name: str = "custom"
    # (dvp, dvs, drho): cell materials uniform in [vp - dvp, vp + dvp] etc. from PETSc's RAND48
    # (SpecFECtxSetPerturbedMaterialProperties_Velocity, se2wave.c:1177-1236)
    perturb: Optional[Tuple[float, float, float]] = None
    # source representation: -1 SeismicSourceCreate's nearest GLL point (the demo's); 0 pointwise,
    # 2 cubic-spline kernel of radius sm_h (<= 0: default), 3 P0 (se2wave.c:2202-2266, -source_impl)
    src_impl: int = -1
    sm_h: float = 0.0
    # interpolating receivers (RecordUV_interp, se2wave.c:2445-2581): u, v (and a, curl v) at the
    # exact points from the Lagrange interpolant of the containing element
    interp_receivers: List[Tuple[float, float]] = field(default_factory=list)

    @property
    def ne(self) -> int:
        return self.mx * self.my

    @property
    def nx_g(self) -> int:
        return self.p * self.mx + 1

    @property
    def ny_g(self) -> int:
        return self.p * self.my + 1

    @property
    def nnodes(self) -> int:
        return self.nx_g * self.ny_g

    @property
    def ndof(self) -> int:
        return 2 * self.nnodes

    def replace(self, **kw) -> "Spec":
        return dataclasses.replace(self, **kw)

    def cell_arrays(self) -> Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]]:
        """Per-cell (vp, vs, rho) as contiguous float64 arrays, or None when constant."""
        if self.cell_vp is None:
            return None
        ne = self.ne
        vp = np.ascontiguousarray(self.cell_vp, dtype=np.float64).reshape(ne)
        vs = np.ascontiguousarray(self.cell_vs, dtype=np.float64).reshape(ne)
        rho = np.ascontiguousarray(self.cell_rho, dtype=np.float64).reshape(ne)
        return vp, vs, rho

    def to_text(self, cell_file: Optional[str] = None) -> str:
        """Spec file read by the oracle's reference driver."""
        lines = [f"mx {self.mx}", f"my {self.my}", f"p {self.p}",
                 f"scale {self.scale[0]!r} {self.scale[1]!r}", f"shift {self.shift[0]!r} {self.shift[1]!r}",
                 f"vp {self.vp!r}", f"vs {self.vs!r}", f"rho {self.rho!r}",
                 f"cfl {self.cfl!r}", f"dt {self.dt!r}", f"tmax {self.tmax!r}", f"nt {self.nt}"]
        if cell_file:
            lines.append(f"cell_file {cell_file}")
        if self.perturb is not None:
            lines.append("perturb " + " ".join(repr(float(v)) for v in self.perturb))
        for s in self.sources:
            m = " ".join(repr(float(v)) for v in s.moment)
            par = " ".join(repr(float(v)) for v in s.par)
            lines.append(f"src {float(s.x)!r} {float(s.y)!r} {m} {_STF_NAMES[s.stf]} {par}")
        for (x, y) in self.receivers:
            lines.append(f"rec {float(x)!r} {float(y)!r}")
        for (x, y) in self.interp_receivers:   # the reference driver keeps one (RecordUV_interp's static state)
            lines.append(f"irec {float(x)!r} {float(y)!r}")
        return "\n".join(lines) + "\n"


def demo(mx: int = 8, my: Optional[int] = None, p: int = 2, tmax: float = 0.4) -> Spec:
    """The reference demo (se2wave.c:4541-4807) at the given mesh size."""
    M = 1000.0
    return Spec(mx=mx, my=mx if my is None else my, p=p, tmax=tmax, name="demo",
                sources=[Source(0.1, 100.1, (M, 0.0, 0.0, M), STF_RICKER, (0.15, 12.0, 1.0)),
                         Source(400.1, 400.1, (0.0, -M, M, 0.0), STF_RICKER, (0.25, 4.0, 1.0))],
                receivers=[(100.0, 200.0), (150.0, 200.0), (180.0, 200.0)])


def explosion64(mx: int = 64, my: Optional[int] = None, p: int = 6, tmax: float = 0.4) -> Spec:
    """2 km square, homogeneous, explosive source at the centre, receiver at (500, 500)."""
    return Spec(mx=mx, my=mx if my is None else my, p=p, vp=6000.0, vs=3464.0, rho=2700.0,
                cfl=0.2, tmax=tmax, name="explosion64",
                sources=[Source(0.0, 0.0, (1e15, 0.0, 0.0, 1e15), STF_RICKER, (0.15, 10.0, 1.0))],
                receivers=[(500.0, 500.0)])


def grf2048(mx: int = 2048, my: Optional[int] = None, p: int = 4, nt: int = 20000, seed: int = 2048,
            cells: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None) -> Spec:
    """20 km square with a Gaussian-random-field Vp (mean 5000, 10 % std, correlation
    length 8 cells), Vp/Vs = 1.73, rho = 2700; explosive Ricker f0 = 8 Hz source at the
    centre; 64 receivers on the line y = +2500 m, x in [-8000, 8000].  Degree 1 has no
    element-interior GLL point, so there the source and receivers snap to the nearest
    node (the reference's -use_nearest_internal_gll false)."""
    my = mx if my is None else my
    if cells is None:
        from . import host  # C generator in the host library
        vp = host.gaussian_random_field(mx, my, mean=5000.0, rel_std=0.10, corr_cells=8.0, seed=seed)
        cells = (vp, vp / 1.73, np.full_like(vp, 2700.0))
    rec = [(float(x), 2500.0) for x in np.linspace(-8000.0, 8000.0, 64)]
    return Spec(mx=mx, my=my, p=p, scale=(20000.0, 20000.0), shift=(-10000.0, -10000.0),
                vp=5000.0, vs=5000.0 / 1.73, rho=2700.0,
                cell_vp=cells[0], cell_vs=cells[1], cell_rho=cells[2],
                cfl=0.2, tmax=1.0e30, nt=nt, name="grf2048", nearest_internal_gll=(p > 1),
                sources=[Source(0.0, 0.0, (1e15, 0.0, 0.0, 1e15), STF_RICKER, (0.15, 8.0, 1.0))],
                receivers=rec)


def shot(seed: int, index: int, kind: int = 0, nt: Optional[int] = None, p: Optional[int] = None,
         size: Optional[Tuple[int, int]] = None) -> Spec:
    """Shot `index` of the seeded distribution `kind` (0 ensemble, 1 training, 2 out-of-distribution),
    drawn by the host library's C generator.  Domain [0, Lx] x [0, Ly], 31.25 m elements, dt = 0.2 CFL.
    `size` = (mx, my) replaces the drawn mesh, with the geometry scaled along (small test cases)."""
    from . import host
    d = host.shot_draw(seed, index, kind)
    if size is not None:
        fx, fy = size[0] / d.mx, size[1] / d.my
        d.mx, d.my = int(size[0]), int(size[1])
        d.Lx, d.Ly = d.mx * d.h, d.my * d.h
        d.interface_y *= fy
        for i in range(d.ninc):
            d.inc[i][0] *= fx; d.inc[i][1] *= fy; d.inc[i][2] *= fx; d.inc[i][3] *= fy
        d.src_xy[0] *= fx
        d.src_xy[1] *= fy
    vp, vs, rho = host.shot_materials(d)
    Lx, Ly = d.Lx, d.Ly
    yr = Ly - 1.0e-3        # 1 mm below the top surface: the receivers snap to the surface nodes
    rec = [(float(x), float(yr)) for x in np.linspace(0.05 * Lx, 0.95 * Lx, d.nrec)]
    src = Source(float(d.src_xy[0]), float(d.src_xy[1]), tuple(float(m) for m in d.moment), STF_RICKER,
                 (float(d.t0), float(d.f0), 1.0))
    return Spec(mx=d.mx, my=d.my, p=d.p if p is None else p, scale=(Lx, Ly), shift=(0.0, 0.0),
                vp=float(vp.mean()), vs=float(vs.mean()), rho=float(rho.mean()),
                cell_vp=vp, cell_vs=vs, cell_rho=rho, cfl=0.2, tmax=1.0e30,
                nt=int(d.nsteps if nt is None else nt), name=f"shot{kind}_{seed}_{index}",
                sources=[src], receivers=rec)


def ensemble(nshots: int = 256, seed: int = 3, kind: int = 0, nt: Optional[int] = None, first: int = 0) -> List[Spec]:
    """The batched-ensemble workload: `nshots` seeded draws first, first + 1, ... (256 shots,
    5000 steps by default)."""
    return [shot(seed, i, kind, nt) for i in range(first, first + nshots)]


def ensemble_shard(nshots: int, rank: int, seed: int = 3, kind: int = 0, nt: Optional[int] = None) -> List[Spec]:
    """Rank `rank`'s shots of a multi-GPU ensemble: draws rank * nshots ... (rank + 1) * nshots - 1.
    Shots are independent, so every GPU runs its own block of draws with no exchange (weak
    scaling: the work per GPU is fixed)."""
    return ensemble(nshots, seed, kind, nt, first=rank * nshots)
