"""Load the committed golden vectors (tests/golden/*.npz) and the specs they were made from."""
import os

import numpy as np

from se2dr_fork_gb300 import spec as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name: str):
    path = os.path.join(GOLDEN, name + ".npz")
    d = np.load(path, allow_pickle=False)
    return {k: d[k] for k in d.files}


def spec_of(d) -> S.Spec:
    g = lambda k: d["spec_" + k]
    srcs = [S.Source(float(xy[0]), float(xy[1]), tuple(float(x) for x in m), int(t), tuple(float(x) for x in par))
            for xy, m, t, par in zip(g("src_xy"), g("src_m"), g("stf_type"), g("stf_par"))]
    sp = S.Spec(mx=int(g("mx")), my=int(g("my")), p=int(g("p")), scale=tuple(g("scale")), shift=tuple(g("shift")),
                vp=float(g("vp")), vs=float(g("vs")), rho=float(g("rho")), cfl=float(g("cfl")), dt=float(g("dt")),
                tmax=float(g("tmax")), nt=int(g("nt")), nearest_internal_gll=bool(int(g("nearest_internal_gll"))),
                sources=srcs, receivers=[tuple(r) for r in g("rec_xy")])
    if "spec_cell_vp" in d:
        sp = sp.replace(cell_vp=g("cell_vp"), cell_vs=g("cell_vs"), cell_rho=g("cell_rho"))
    if "spec_perturb" in d:
        sp = sp.replace(perturb=tuple(float(x) for x in g("perturb")))
    if "spec_interp_xy" in d:
        sp = sp.replace(interp_receivers=[tuple(float(v) for v in r) for r in g("interp_xy")])
    return sp


def names(prefix: str):
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith(prefix) and f.endswith(".npz"))


# ---------------------------------------------------------------- FP32 tolerances
# Relative L2 error bars per trace component (ux uy vx vy ax ay curl) of the FAST FP32
# modes (plain and Kahan-compensated) against FP64.  These modes do NOT meet the 1e-5
# bar on every trace: it holds for displacement, while acceleration and curl(v) are
# second and first spatial derivatives of an FP32-rounded field, which the stiffness
# operator amplifies by ~(p^2 lambda / 2 pi h)^2 and ~(p^2 lambda / 2 pi h).  The
# two-float mode (fp32_df) meets 1e-5 on every component (tests/test_fp32_df.py).
FP32_COMPONENT_TOL = (1e-5, 1e-5, 1e-4, 1e-4, 5e-3, 5e-3, 5e-3)
# curl(v) is compared on the scale of the velocity gradient, k |v| with the shear
# wavenumber of the source's peak frequency: an explosive source radiates P waves,
# whose curl is pure discretisation noise (1e-11 k|v| in FP64), so a relative
# error of the curl itself would not measure anything.
K_SHEAR = 2.0 * np.pi * 10.0 / 3464.0


def fp32_errors(tr32, tr64, k=K_SHEAR):
    errs = [rel_l2(tr32[:, 1 + c::7], tr64[:, 1 + c::7]) for c in range(6)]
    v = tr64[:, 3::7], tr64[:, 4::7]
    scale = max(np.linalg.norm(tr64[:, 7::7]), k * np.sqrt(np.linalg.norm(v[0]) ** 2 + np.linalg.norm(v[1]) ** 2))
    errs.append(np.linalg.norm(tr32[:, 7::7] - tr64[:, 7::7]) / scale)
    return errs


def fp32_errors_ok(tr32, tr64, k=K_SHEAR):
    errs = fp32_errors(tr32, tr64, k)
    return all(e <= t for e, t in zip(errs, FP32_COMPONENT_TOL)), errs


def rel_l2(x, ref):
    den = np.linalg.norm(ref)
    return np.linalg.norm(x - ref) / (den if den > 0 else 1.0)


def read_vts(path):
    """Arrays of a VTK XML StructuredGrid file with raw appended data (UInt64 headers)."""
    import re
    blob = open(path, "rb").read()
    head, _, tail = blob.partition(b"<AppendedData encoding=\"raw\">")
    data = tail[tail.index(b"_") + 1:]
    ext = [int(v) for v in re.search(rb'WholeExtent="([^"]+)"', head).group(1).split()]
    out = {}
    for m in re.finditer(rb'<DataArray type="Float64" Name="([^"]+)" NumberOfComponents="(\d)" format="appended" '
                         rb'offset="(\d+)"', head):
        name, nc, off = m.group(1).decode(), int(m.group(2)), int(m.group(3))
        nbytes = int(np.frombuffer(data[off:off + 8], dtype=np.uint64)[0])
        out[name] = np.frombuffer(data[off + 8:off + 8 + nbytes], dtype=np.float64).reshape(-1, nc)
    return (ext[1] + 1, ext[3] + 1), out
