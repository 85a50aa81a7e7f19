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
    return sp


def names(prefix: str):
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith(prefix) and f.endswith(".npz"))
