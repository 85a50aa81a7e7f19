"""Surrogate pipeline pieces that need the GPU: solver traces of mirrored
problems (the augmentation's premise), a short end-to-end train/predict, and what
a trained network gains over the method without it (the coarse-solver ladder) at
equal misfit."""
import time

import numpy as np
import pytest

from se2dr_fork_gb300 import spec as S
from se2dr_fork_gb300 import surrogate as SU

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _libs(gpu_lib, nn_lib):
    return gpu_lib, nn_lib


def mirror_spec(sp: S.Spec) -> S.Spec:
    flip = lambda a: np.ascontiguousarray(np.asarray(a).reshape(sp.my, sp.mx)[:, ::-1].reshape(-1))
    src = sp.sources[0]
    Lx = sp.mx * SU.CELL
    return sp.replace(cell_vp=flip(sp.cell_vp), cell_vs=flip(sp.cell_vs), cell_rho=flip(sp.cell_rho),
                      sources=[S.Source(Lx - src.x, src.y, src.moment, src.stf, src.par)])


def test_mirrored_problem_gives_mirrored_traces():
    sp = SU.draw_spec(7, 3)
    traces, _ = SU.solve([sp, mirror_spec(sp)], chunk=2)
    a = traces[0].reshape(16, 2, SU.NSAMP)
    b = traces[1].reshape(16, 2, SU.NSAMP)
    scale = np.abs(a).max()
    assert scale > 1e-12
    assert np.max(np.abs(b[::-1, 0] + a[:, 0])) < 1e-4 * scale
    assert np.max(np.abs(b[::-1, 1] - a[:, 1])) < 1e-4 * scale


def test_short_training_run_fits_and_predicts():
    ds = SU.generate(11, 64)
    data = SU.DeviceData(ds, augment=True)
    assert data.n == 128
    net, st = SU.train(data, np.arange(data.n), SU.receiver_cells(ds.specs[0]), seed=0, epochs=6, batch=32, lr=2e-3)
    assert st["loss"][-1] < st["loss"][0]
    preds = SU.predict([net], data, np.arange(8))
    assert preds.shape == (1, 8, 16, 2048) and np.all(np.isfinite(preds))


def test_solver_ladder_and_equal_misfit():
    """The coarse-solver ladder behind the comparison at equal misfit: the fine configuration
    itself reproduces the draws' traces exactly, coarser ones cost less per draw and miss more."""
    specs = SU.specs_of(21, 3)
    true, _ = SU.solve(specs, chunk=3)
    lad = SU.solver_ladder(specs, true, ladder=[(SU.GRID, 4), (64, 4), (32, 2)])
    fine, mid, coarse = lad
    assert fine["dt_ratio"] == 1 and fine["misfit_mean"] == 0.0
    assert mid["dt_ratio"] == 2 and coarse["dt_ratio"] == 4
    assert 0.0 < mid["misfit_mean"] < coarse["misfit_mean"] and np.isfinite(coarse["misfit_mean"])
    assert coarse["nodes"] < mid["nodes"] < fine["nodes"]
    eq = SU.equal_misfit(lad, mid["misfit_mean"], 1.0)
    assert eq["solver"]["misfit_mean"] <= mid["misfit_mean"] and eq["gain"] == 1.0 / eq["solver"]["draws_per_s"]
    assert eq["gain_solver_time"] <= eq["gain"]      # the solver's device time is at most its wall time
    assert SU.equal_misfit(lad, -1.0, 1.0) == {"solver": None, "gain": None, "gain_solver_time": None}


def test_inference_copies_predict_the_same():
    """Networks re-created for larger inference batches (for_inference) carry the same
    parameters and give the same predictions as the trained ones, whatever the batch."""
    specs = SU.specs_of(31, 6)
    mats, src = SU.inputs_of(specs)
    ds = SU.Dataset(mats, src, np.zeros((6, SU.NREC, 2 * SU.NSAMP), dtype=np.float32), np.zeros(6), specs=specs)
    data = SU.DeviceData(ds, scale=1.0)
    from se2dr_fork_gb300 import nn as N
    net = N.Network(SU.net_config(4), seed=3)
    net.set_receivers(SU.receiver_cells(specs[0]))
    big = SU.for_inference([net], max_batch=8)
    assert big[0].cfg.max_batch == 8 and np.array_equal(big[0].params(), net.params())
    a = SU.predict([net], data, np.arange(6))            # passes of 4 + 2
    b = SU.predict(big, data, np.arange(6))              # one pass of 6
    assert np.array_equal(a, b)


def test_trained_network_beats_the_solver_ladder_at_equal_misfit():
    """The learned part against the method without it: a network trained by the project's
    own kernels (2400 draws and their mirrors, 16 epochs) predicts 64 held-out draws faster
    than the fastest coarse solver of the ladder whose mean misfit is at most the
    network's, against that solver's wall time and against its device time alone."""
    tr = SU.generate(41, 2400)
    te = SU.generate(42, 64)
    dtrain = SU.DeviceData(tr, augment=True)
    dtest = SU.DeviceData(te, scale=dtrain.scale)
    rec_x = SU.receiver_cells(tr.specs[0])
    net, st = SU.train(dtrain, np.arange(dtrain.n), rec_x, seed=0, epochs=16, batch=32, lr=1e-3)
    assert st["loss"][-1] < 0.7 * st["loss"][0]
    inf = SU.for_inference([net], 64)
    SU.predict(inf, dtest, np.arange(8))           # warm: streams and buffers
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    preds = SU.predict(inf, dtest, np.arange(dtest.n))
    secs = time.perf_counter() - t0
    mis = float(SU.rel_l2(preds[0], te.traces).mean())
    lad = SU.solver_ladder(te.specs, te.traces)
    eq = SU.equal_misfit(lad, mis, dtest.n / secs)
    print(f"network misfit {mis:.3f}, {dtest.n / secs:.0f} draws/s; fastest solver at most as wrong: "
          f"{eq['solver'] and (eq['solver']['mx'], eq['solver']['p'], round(eq['solver']['misfit_mean'], 3), round(eq['solver']['draws_per_s']))}; "
          f"gain {eq['gain']}, against its device time {eq['gain_solver_time']}")
    assert 0.0 < mis < 1.0
    assert eq["solver"] is not None, lad
    assert eq["gain"] > 1.0 and eq["gain_solver_time"] > 1.0, eq
