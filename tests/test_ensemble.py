"""Batched ensemble (se2gpu_ensemble_*): many shots of uneven size and degree in
one persistent launch per degree group, blocks of steps replayed as CUDA graphs.

Each shot must evolve bit-identically to a single-shot solver of the same
problem (same FP32 arithmetic, different scheduling); one sample is checked
against the FP64 oracle within the FP32 error bars.
"""
import numpy as np
import pytest

from golden_util import fp32_errors_ok
from oracle import oracle as O
from se2dr_fork_gb300 import gpu as G
from se2dr_fork_gb300 import host as H
from se2dr_fork_gb300 import spec as S

pytestmark = pytest.mark.gpu

SIZES = [(8, 8), (13, 21), (24, 9), (17, 17), (30, 11), (9, 26), (1, 1)]
DEGREES = [3, 4, 6, 3, 4, 6, 4]


@pytest.fixture(scope="module", autouse=True)
def _lib(gpu_lib):
    return gpu_lib


def small_setups(seed=7, nt=64, n=len(SIZES)):
    return [H.Setup(S.shot(seed, i, size=SIZES[i], p=DEGREES[i], nt=nt)) for i in range(n)]


def single_runs(setups, precision, chunks, configs):
    out = []
    for su in setups:
        sol = G.Solver(su, precision)
        sol.set_tile_config(configs[su.p])
        tr = np.concatenate([sol.run(n) for n in chunks], axis=0)
        out.append((tr, *sol.fields()))
        sol.close()
    return out


def ensemble_runs(ens, chunks):
    trs = [ens.advance(n) for n in chunks]
    return [(np.concatenate([t[i] for t in trs], axis=0), *ens.fields(i)) for i in range(len(ens))]


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("precision", ["fp32_kahan", "fp32"])
def test_ensemble_bitwise_equals_single_shot_solvers(precision):
    setups = small_setups()
    ens = G.Ensemble(setups, precision, block=4)
    chunks = [11, 5, 4]          # graph blocks, an odd remainder (buffer parity flips), the other parity's graph
    got = ensemble_runs(ens, chunks)
    info = ens.info()
    assert info["shots"] == len(setups) and info["groups"] == 3
    assert info["replays"] == 2 + 1 + 1
    configs = {p: ens.tile_config(p) for p in ens.degrees()}
    ref = single_runs(setups, precision, chunks, configs)
    for i, (g, r) in enumerate(zip(got, ref)):
        assert g[0].shape == (20, 1 + 7 * setups[i].nrec)
        assert same(g, r), f"shot {i} (p={setups[i].p}, {setups[i].mx}x{setups[i].my})"


def test_ensemble_graphs_and_plain_launches_agree():
    setups = small_setups(seed=11, n=6)
    runs = []
    for graphs in (True, False):
        ens = G.Ensemble(setups, "fp32_kahan", block=6)
        ens.set_graphs(graphs)
        runs.append(ensemble_runs(ens, [13, 6]))
        assert (ens.info()["replays"] > 0) == graphs
        ens.close()
    for a, b in zip(*runs):
        assert same(a, b)


def test_ensemble_tile_configs_agree():
    setups = small_setups(seed=5, n=6)
    ens0 = G.Ensemble(setups, "fp32_kahan", block=4)
    ref = ensemble_runs(ens0, [9])
    ens1 = G.Ensemble(setups, "fp32_kahan", block=4)
    for p in ens1.degrees():
        ens1.set_tile_config(p, 1)
        assert ens1.tile_config(p) == 1
    got = ensemble_runs(ens1, [9])
    for a, b in zip(got, ref):
        assert same(a, b)


def test_ensemble_set_fields_matches_single_solver():
    setups = small_setups(seed=2, n=3)
    rng = np.random.default_rng(0)
    ens = G.Ensemble(setups, "fp32_kahan", block=4)
    inits = []
    for i, su in enumerate(setups):
        u0, v0 = rng.standard_normal(su.ndof) * 1e-6, rng.standard_normal(su.ndof) * 1e-4
        ens.set_fields(i, u0, v0, np.zeros(su.ndof))
        inits.append((u0, v0))
    got = ensemble_runs(ens, [7])
    for i, su in enumerate(setups):
        sol = G.Solver(su, "fp32_kahan")
        sol.set_tile_config(ens.tile_config(su.p))
        sol.set_fields(*inits[i], np.zeros(su.ndof))
        assert same(got[i], (sol.run(7), *sol.fields()))


def test_ensemble_sample_vs_fp64_oracle():
    """Two shots of the ensemble distribution, FP32-Kahan in the batch, against the FP64 oracle."""
    specs = [S.shot(3, 0, size=(14, 11), nt=400), S.shot(3, 1, size=(10, 13), nt=400)]
    ens = G.Ensemble([H.Setup(sp) for sp in specs], "fp32_kahan", block=50)
    trs = ens.advance(400)
    for sp, tr in zip(specs, trs):
        rr = O.OracleSolver(sp).run(400)["traces"]
        assert np.array_equal(tr[:, 0], rr[:, 0])
        k = 2.0 * np.pi * sp.sources[0].par[1] / float(np.min(sp.cell_vs))
        ok, errs = fp32_errors_ok(tr, rr, k)
        print(sp.name, ["%.2e" % e for e in errs])
        assert ok, errs


def test_ensemble_errors():
    su = small_setups(n=1)
    with pytest.raises(G.GpuError, match="FP32"):
        G.Ensemble(su, "fp64")
    with pytest.raises(G.GpuError, match="block"):
        G.Ensemble(su, "fp32", block=0)
    ens = G.Ensemble(su, "fp32", block=2)
    with pytest.raises(G.GpuError, match="degree"):
        ens.set_tile_config(5, 0)
    with pytest.raises(G.GpuError, match="shot"):
        ens.fields(3)


def test_group_larger_than_one_launch():
    """A degree group of more shots than one launch carries (SE2P_BATCH_SHOTS = 96) runs as
    several launches per step; shots in the first and the last launch stay bit-identical to
    single-shot solvers."""
    n = 100
    setups = [H.Setup(S.shot(11, i, size=(3 + i % 5, 2 + i % 4), p=3, nt=24)) for i in range(n)]
    ens = G.Ensemble(setups, "fp32_kahan", block=4)
    got = ensemble_runs(ens, [9])
    info = ens.info()
    assert info["groups"] == 1 and info["launches"] == 2 * 9 + 3   # 2 launches per step + 3 receiver kernels
    cfg = {3: ens.tile_config(3)}
    for i in (0, 50, 95, 96, 99):
        ref = single_runs([setups[i]], "fp32_kahan", [9], cfg)[0]
        assert same(got[i], ref), i
    ens.close()
