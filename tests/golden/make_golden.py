"""Generate the golden vectors in tests/golden/ from the reference itself.

The reference (se2wave.c) is compiled in place, unmodified, against the
petsclite shim (oracle/Makefile target ``ref``) and driven by
oracle/ref_driver.c, which calls the reference's own set-up, element loop,
source, STF and receiver routines.  Receiver values are captured from the
reference's own fprintf calls at full precision.

Run here (where the reference tree exists):  python tests/golden/make_golden.py
Outputs: tests/golden/*.npz (committed), never read at run time by the product.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from se2dr_fork_gb300 import spec as S  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def hetero(p: int, mx: int = 7, my: int = 5, nt: int = 60, seed: int = 100) -> S.Spec:
    """Small heterogeneous mesh, three sources (one per STF kind), five receivers
    (including domain corners and the source point), fixed step count."""
    rng = np.random.default_rng(seed + p)
    return S.explosion64(mx, my, p=p, tmax=1.0).replace(
        nt=nt, nearest_internal_gll=(p > 1), name=f"hetero_p{p}",
        cell_vp=rng.uniform(5000, 7000, mx * my), cell_vs=rng.uniform(2800, 3500, mx * my),
        cell_rho=rng.uniform(2000, 3000, mx * my),
        sources=[S.Source(13.7, -200.0, (1e15, 3e14, -2e14, 5e14), S.STF_RICKER, (0.01, 30.0, 1.0)),
                 S.Source(-300.0, 100.0, (0.0, 1e14, 1e14, 0.0), S.STF_GAUSSIAN, (0.005, 300.0, 2.0)),
                 S.Source(250.0, 250.0, (1e14, 0.0, 0.0, 1e14), S.STF_YOFFE, (0.0015, 0.006, 1.1))],
        receivers=[(500.0, 500.0), (-1000.0, -1000.0), (1000.0, 1000.0), (0.0, 0.0), (-999.9, 403.2)])


def ragged() -> S.Spec:
    """A mesh that is not a multiple of any tile edge, sources straddling tile seams."""
    return S.explosion64(13, 9, p=4, tmax=1.0).replace(
        nt=40, name="ragged_p4",
        sources=[S.Source(-384.6, -111.1, (1e15, 0.0, 0.0, 1e15), S.STF_RICKER, (0.01, 25.0, 1.0)),
                 S.Source(230.77, 0.0, (0.0, -1e15, 1e15, 0.0), S.STF_RICKER, (0.012, 20.0, 1.0))],
        receivers=[(230.77, 0.0), (-384.6, 333.3), (999.0, -999.0)])


def save(name: str, **arrays):
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"  wrote {os.path.relpath(path, ROOT)} ({os.path.getsize(path) / 1024:.1f} KiB)")


def spec_arrays(sp: S.Spec) -> dict:
    """The spec itself, so the tests rebuild exactly the same problem."""
    d = dict(mx=sp.mx, my=sp.my, p=sp.p, scale=np.array(sp.scale), shift=np.array(sp.shift),
             vp=sp.vp, vs=sp.vs, rho=sp.rho, cfl=sp.cfl, dt=sp.dt, tmax=sp.tmax, nt=sp.nt,
             nearest_internal_gll=int(sp.nearest_internal_gll),
             src_xy=np.array([[s.x, s.y] for s in sp.sources]).reshape(-1, 2),
             src_m=np.array([s.moment for s in sp.sources]).reshape(-1, 4),
             stf_type=np.array([s.stf for s in sp.sources], dtype=np.int32),
             stf_par=np.array([s.par for s in sp.sources]).reshape(-1, 3),
             rec_xy=np.array(sp.receivers, dtype=np.float64).reshape(-1, 2))
    if sp.cell_vp is not None:
        d.update(cell_vp=np.asarray(sp.cell_vp), cell_vs=np.asarray(sp.cell_vs), cell_rho=np.asarray(sp.cell_rho))
    if sp.perturb is not None:
        d.update(perturb=np.array(sp.perturb, dtype=np.float64))
    if sp.interp_receivers:
        d.update(interp_xy=np.array(sp.interp_receivers, dtype=np.float64).reshape(-1, 2))
    return {"spec_" + k: v for k, v in d.items()}


def source_vectors():
    """Assembled source vectors of the alternative source representations (se2wave.c:1716-2200)."""
    for p in (2, 4, 6):
        sp = S.demo(9, 7, p=p, tmax=1.0).replace(nt=5, name=f"srcvec_p{p}",
                                                  sources=[S.Source(137.3, -251.9, (1e15, 3e14, -2e14, 5e14))])
        out = {f"g_impl{i}": O.ref_source_vector(sp, i) for i in (0, 2, 3)}
        out["g_impl2_h310p5"] = O.ref_source_vector(sp, 2, ["-sm_h", "310.5"])
        save(f"srcvec_p{p}", **out, **spec_arrays(sp))


def perturbed():
    """SpecFECtxSetPerturbedMaterialProperties_Velocity (se2wave.c:1177-1236) on the demo."""
    sp = S.demo(9, 7, p=3, tmax=1.0).replace(nt=60, perturb=(500.0, 200.0, 100.0), name="perturbed_p3")
    r = O.ref_run(sp)
    if r["returncode"] != 0:
        raise RuntimeError(r["stderr"])
    res = run_case(sp, fields=True)
    save("perturbed_p3", cell_lmr=r["cell_lmr"], **res, **spec_arrays(sp))


def interp():
    """Interpolating receiver RecordUV_interp (se2wave.c:2445-2581) on a heterogeneous mesh,
    p = 3 and 4, one point inside an element and one on an element edge (xi = -1)."""
    for p, xy in ((3, (137.3, -251.9)), (4, (-250.0, 311.7))):
        rng = np.random.default_rng(40 + p)
        mx, my = 9, 7
        sp = S.demo(mx, my, p=p, tmax=1.0).replace(
            nt=50, name=f"interp_p{p}", interp_receivers=[xy],
            cell_vp=rng.uniform(5000, 7000, mx * my), cell_vs=rng.uniform(2800, 3500, mx * my),
            cell_rho=rng.uniform(2000, 3000, mx * my))
        r = O.ref_run(sp)
        if r["returncode"] != 0:
            raise RuntimeError(r["stderr"])
        fname = f"defaultsource-receiver-{mx}x{my}-p{p}.dat"
        save(f"interp_p{p}", interp=r["interp"], interp_xri_text=r["interp_xri_text"], traces=r["traces"],
             u=r["u"], v=r["v"], dat_name=np.array(fname), dat_text=np.array(r[fname]), **spec_arrays(sp))


def run_case(sp: S.Spec, fields: bool, extra=()):
    t0 = time.time()
    r = O.ref_run(sp, extra_args=list(extra))
    if r["returncode"] != 0:
        raise RuntimeError(f"reference failed on {sp.name}: {r['stderr'][-2000:]}")
    out = dict(traces=r["traces"], D=r["D"], xi=r["xi"], w1d=r["w1d"], dt_cfl=r["dt_cfl"],
               run_meta=r["run_meta"], src_values=r["src_values"], src_index=r["src_index"])
    if fields:
        out.update(u=r["u"], v=r["v"], a=r["a"], mass=r["mass"], coords=r["coords"])
    norms = [list(map(float, l.split())) for l in r["norms.txt"].splitlines() if l.strip()]
    out["norms"] = np.array(norms).reshape(-1, 7)
    dat = [k for k in r if k.endswith(".dat")]
    if dat:
        out["dat_text"] = np.array(r[dat[0]])
    print(f"  {sp.name}: {r['traces'].shape[0]} steps in {time.time() - t0:.1f}s")
    return out


def reference_main_outputs(args, name):
    """stdout, .dat and .mpimeta of the reference's own main() (se2wave.c:4916-4951)."""
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([O.REF_DRIVER, "demo", *args], cwd=d, capture_output=True, text=True, check=True)
        files = {f: open(os.path.join(d, f)).read() for f in sorted(os.listdir(d))}
    out = {"args": np.array(args), "stdout": np.array(r.stdout)}
    for f, text in files.items():
        out["file_" + f.replace(".", "_").replace("-", "_")] = np.array(text)
        out["name_" + f.replace(".", "_").replace("-", "_")] = np.array(f)
    save(name, **out)


def main():
    if "--perturbed-only" in sys.argv:
        O.build_ref()
        perturbed()
        source_vectors()
        return
    if "--interp-only" in sys.argv:
        O.build_ref()
        interp()
        return
    if "--cli-only" in sys.argv:
        O.build_ref()
        reference_main_outputs([], "cli_demo_default")
        reference_main_outputs(["-mx", "6", "-my", "4", "-bdegree", "3", "-tmax", "0.1"], "cli_demo_6x4_p3")
        return
    if not O.build_ref():
        sys.exit("the reference tree is not available; golden vectors can only be generated where it is")
    O.build()
    print("basis tables (CreateGLLCoordsWeights / TabulateBasisDerivatives1d_CLEGENDRE), p = 1..8")
    for p in range(1, 9):
        sp = hetero(p)
        extra = [] if p > 1 else ["-use_nearest_internal_gll", "false"]
        res = run_case(sp, fields=p in (1, 2, 5, 8), extra=extra)
        save(f"hetero_p{p}", **res, **spec_arrays(sp))
    sp = ragged()
    save("ragged_p4", **run_case(sp, fields=True), **spec_arrays(sp))
    sp = S.demo(8, p=2)
    save("demo8_p2", **run_case(sp, fields=True), **spec_arrays(sp))

    perturbed()
    source_vectors()
    interp()

    print("internal force AssembleLinearForm_ElastoDynamics2d on random displacements")
    for p, mx, my in [(1, 6, 5), (3, 6, 5), (4, 9, 10), (7, 3, 4)]:
        sp = S.explosion64(mx, my, p=p).replace(name=f"force_p{p}", nearest_internal_gll=False,
                                                sources=[], receivers=[])
        rng = np.random.default_rng(7 + p)
        u = rng.standard_normal(sp.ndof)
        r = O.ref_run(sp, force_u=u)
        if r["returncode"] != 0:
            raise RuntimeError(r["stderr"])
        save(f"force_p{p}", u=u, force=r["force"], **spec_arrays(sp))

    print("source-time functions (SeismicSTFEvaluate_*)")
    stf = {}
    stf["ricker"] = O.ref_stf("ricker", 0.15, 12.0, 1.0, 0.0, 1.0e-3, 2000)
    stf["gaussian"] = O.ref_stf("gaussian", 0.2, 40.0, 3.0, 0.0, 1.0e-3, 2000)
    stf["yoffe_mode1"] = O.ref_stf("yoffe", 0.15, 1.0, 1.1, -0.01, 1.0e-3, 1400)
    stf["yoffe_mode2"] = O.ref_stf("yoffe", 0.3, 0.45, 1.1, -0.01, 1.0e-3, 1200)
    save("stf", **stf)

    print("explosion64: 64x64 elements, degree 6, dt = 0.2 CFL, tmax 0.4 s (full run)")
    sp = S.explosion64()
    res = run_case(sp, fields=False)
    save("explosion64", traces=res["traces"], run_meta=res["run_meta"], dt_cfl=res["dt_cfl"], norms=res["norms"],
         **spec_arrays(sp))

    print("README demo (se2wave.app -mx 64 -my 64 -bdegree 6 -tmax 0.4): receiver 0 vy")
    sp = S.demo(64, p=6)
    res = run_case(sp, fields=False)
    tr = res["traces"]
    save("readme_demo64", time=tr[:, 0], vy0=tr[:, 4], run_meta=res["run_meta"])

    print("the reference executable's own output (main)")
    reference_main_outputs([], "cli_demo_default")
    reference_main_outputs(["-mx", "6", "-my", "4", "-bdegree", "3", "-tmax", "0.1"], "cli_demo_6x4_p3")


if __name__ == "__main__":
    main()
