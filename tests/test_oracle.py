"""The oracle port (oracle/se2_oracle.c) against golden vectors produced by the
reference itself (se2wave.c compiled in place; tests/golden/make_golden.py).

On x86-64 -- where the golden vectors were made -- the port must match bit for
bit.  On other hosts libm may round a transcendental differently in the last
place, so there the bar is the FP64 parity tolerance, 1e-12 relative L2.
"""
import platform

import numpy as np
import pytest

from golden_util import load, spec_of
from oracle import oracle as O

BITWISE = platform.machine() in ("x86_64", "AMD64")


def same(x, ref, tol=1e-12):
    if BITWISE:
        return np.array_equal(x, ref)
    den = np.linalg.norm(ref)
    return np.linalg.norm(np.asarray(x) - ref) <= tol * (den if den > 0 else 1.0)


@pytest.mark.parametrize("p", range(1, 9))
def test_oracle_heterogeneous_runs(p):
    d = load(f"hetero_p{p}")
    o = O.OracleSolver(spec_of(d))
    assert same(o.get("D"), d["D"]) and same(o.get("xi"), d["xi"]) and same(o.get("w1d"), d["w1d"])
    assert same(o.get("src_values"), d["src_values"])
    assert np.array_equal(o.get("src_index").astype(np.int32), d["src_index"])
    assert same(np.array([o.dt_cfl]), d["dt_cfl"])
    r = o.run(10 ** 6, norms=True)
    assert r["traces"].shape == d["traces"].shape
    for c in range(d["traces"].shape[1]):
        assert same(r["traces"][:, c], d["traces"][:, c])
    if "u" in d:
        u, v, a = o.state()
        assert same(u, d["u"]) and same(v, d["v"]) and same(a, d["a"])
        assert same(o.get("mass"), d["mass"]) and same(o.get("coords"), d["coords"])


@pytest.mark.parametrize("name", ["ragged_p4", "demo8_p2"])
def test_oracle_fields(name):
    d = load(name)
    o = O.OracleSolver(spec_of(d))
    r = o.run(10 ** 6)
    assert same(r["traces"], d["traces"])
    u, v, a = o.state()
    assert same(u, d["u"]) and same(v, d["v"]) and same(a, d["a"])


@pytest.mark.parametrize("p", [1, 3, 4, 7])
def test_oracle_internal_force(p):
    d = load(f"force_p{p}")
    o = O.OracleSolver(spec_of(d))
    assert same(o.force(d["u"]), d["force"])


@pytest.mark.parametrize("kind,typ,par,t0,n", [("ricker", 0, (0.15, 12.0, 1.0), 0.0, 2000),
                                               ("gaussian", 1, (0.2, 40.0, 3.0), 0.0, 2000),
                                               ("yoffe_mode1", 2, (0.15, 1.0, 1.1), -0.01, 1400),
                                               ("yoffe_mode2", 2, (0.3, 0.45, 1.1), -0.01, 1200)])
def test_oracle_stf(kind, typ, par, t0, n):
    g = load("stf")[kind]
    v = O.stf(typ, par, t0, 1.0e-3, n)
    assert same(v, g[:, 1])


def test_oracle_demo_text_output_matches_reference_dat():
    """The reference's own .dat rows are the oracle's values printed with its formats."""
    d = load("demo8_p2")
    text = str(d["dat_text"])
    rows = [l for l in text.splitlines() if not l.startswith("#")]
    o = O.OracleSolver(spec_of(d))
    tr = o.run(10 ** 6)["traces"]
    for line, row in zip(rows, tr):
        vals = ["%1.4e" % row[0]] + ["%+1.8e" % x for x in row[1:]]
        assert line.split() == vals


def test_readme_figure_pinned():
    """Receiver-0 vy of the README run (docs/figs/se2wave-demo-vy.png, README.md:42-49),
    from the reference compiled in place: the features read off the published plot."""
    d = load("readme_demo64")
    t, vy = d["time"], d["vy0"]
    feats = [((0.11, 0.145), "min", -1.3e-9, 0.13), ((0.145, 0.175), "max", 5.2e-9, 0.16),
             ((0.175, 0.2), "min", -6.0e-9, 0.187), ((0.2, 0.23), "max", 3.0e-9, 0.215),
             ((0.28, 0.36), "min", -2.9e-9, 0.32)]
    for (lo, hi), kind, val, when in feats:
        m = (t > lo) & (t < hi)
        i = vy[m].argmax() if kind == "max" else vy[m].argmin()
        assert abs(vy[m][i] - val) < 0.15e-9, (lo, hi, vy[m][i])
        assert abs(t[m][i] - when) < 0.006
    assert np.abs(vy[t < 0.09]).max() < 1e-10  # flat until the P wave arrives
    assert abs(vy[-1] - 3.5e-9) < 0.2e-9


def test_oracle_errors():
    from se2dr_fork_gb300 import spec as S
    with pytest.raises(RuntimeError):  # source outside the domain (se2wave.c:3013-3016)
        O.OracleSolver(S.demo(4).replace(sources=[S.Source(5000.0, 0.0, (1, 0, 0, 1))]))
    with pytest.raises(RuntimeError):  # degree 1 with the interior-GLL source rule (3128-3130)
        O.OracleSolver(S.demo(4, p=1))
    with pytest.raises(RuntimeError):  # receiver outside the domain (2727-2730)
        O.OracleSolver(S.demo(4).replace(receivers=[(0.0, 1e6)]))
