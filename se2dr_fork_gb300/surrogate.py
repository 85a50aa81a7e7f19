"""Neural-operator surrogate of the se2wave solver: training data from the
batched FP32 solver, training and inference with the network kernels of
libse2nn.so, and serving with an ensemble-disagreement gate and solver fallback.

Workload (fixed here because the task leaves it open):
* draws of the layered + elliptical-inclusion material distribution on a 4 km
  square, 128 x 128 elements of degree 4 (host generator, kind SHOT_TRAINING;
  SHOT_OOD for out-of-distribution requests: Vp up to 7500 m/s, two inclusions);
* one explosive source (M = diag(1e15, 1e15)) with a Ricker wavelet of 5 Hz
  (t0 = 0.3 s; the low end of the ensemble's 5-20 Hz range) at a random
  position in the lower half -- the network's inputs are the materials and the
  source position only, so the mechanism and the wavelet are the same for every
  draw.  The network reads each receiver's trace along its grid column (128
  rows for 1.47 s), and its 16 retained modes resolve about 10.9 Hz along that
  axis, which holds most of a 5 Hz Ricker wavelet's spectrum;
* one time step for every draw: 0.5 x the CFL step of Vp = 7500 m/s on these
  elements (0.4 CFL at the in-distribution maximum of 6000 m/s), 4096 steps;
* targets: the velocity (vx, vy) at 16 surface receivers, every 4th step:
  16 x 2 x 1024 samples per draw, scaled by one global factor.
"""
from __future__ import annotations

import concurrent.futures as cf
import dataclasses
import time
from typing import List, Optional

import numpy as np

from . import gpu as G
from . import host as H
from . import nn as N
from . import spec as S

NSTEPS = 4096
DECIMATE = 4
NSAMP = NSTEPS // DECIMATE
NREC = 16
CELL = 31.25
GRID = 128
SIGMA_CELLS = 2.0


def surrogate_dt() -> float:
    """0.5 x the reference's CFL step for Vp = 7500 m/s on 31.25 m elements of degree 4."""
    sp = S.Spec(mx=GRID, my=GRID, p=4, scale=(GRID * CELL, GRID * CELL), shift=(0.0, 0.0), vp=7500.0,
                vs=7500.0 / 1.6, rho=2500.0, cfl=0.5, tmax=1.0e30, nt=1)
    return H.Setup(sp).dt


def draw_spec(seed: int, index: int, kind: int = H.SHOT_TRAINING, dt: Optional[float] = None) -> S.Spec:
    sp = S.shot(seed, index, kind, nt=NSTEPS)
    src = sp.sources[0]
    return sp.replace(dt=surrogate_dt() if dt is None else dt,
                      sources=[S.Source(src.x, src.y, (1e15, 0.0, 0.0, 1e15), S.STF_RICKER, (0.3, 5.0, 1.0))])


def receiver_cells(sp: S.Spec) -> np.ndarray:
    return np.array([min(GRID - 1, int(x / CELL)) for (x, _) in sp.receivers], dtype=np.int32)


@dataclasses.dataclass
class Dataset:
    materials: np.ndarray     # [n, 128, 128, 3] float32 (vp, vs, rho) per cell, row y from the bottom
    src: np.ndarray           # [n, 2] float32 source position in cells (x, y)
    traces: np.ndarray        # [n, 16, 2 * 1024] float32 (vx then vy per receiver)
    kind: np.ndarray          # [n] draw kind
    seconds: float = 0.0      # solver time spent producing it (batched solver, excluding host set-up)
    wall_seconds: float = 0.0  # wall time of the whole solve, host set-up included
    specs: Optional[list] = None

    def __len__(self):
        return self.materials.shape[0]


def _traces_from_rows(rows: np.ndarray, decimate: int = DECIMATE) -> np.ndarray:
    """[steps, 1 + 7 nrec] receiver rows -> [nrec, 2 * NSAMP] velocities every decimate-th step."""
    sel = rows[decimate - 1::decimate, 1:].reshape(-1, NREC, 7)[:NSAMP]
    return np.concatenate([sel[:, :, 2].T, sel[:, :, 3].T], axis=1).astype(np.float32)


def solve(specs: List[S.Spec], precision: str = "fp32_kahan", chunk: int = 1000, block: int = 128,
          threads: int = 16, nsteps: int = NSTEPS, decimate: int = DECIMATE):
    """Solve the draws with the batched FP32 solver; returns ([n, 16, 2048] traces, solver seconds)."""
    out = np.zeros((len(specs), NREC, 2 * NSAMP), dtype=np.float32)
    secs = 0.0
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for c0 in range(0, len(specs), chunk):
            part = specs[c0:c0 + chunk]
            setups = list(ex.map(H.Setup, part))
            t0 = time.perf_counter()
            ens = G.Ensemble(setups, precision, block=block)
            rows = ens.advance(nsteps)
            ens.close()
            secs += time.perf_counter() - t0
            for i, r in enumerate(rows):
                out[c0 + i] = _traces_from_rows(r, decimate)
            del setups, rows
    return out, secs


def specs_of(seed: int, n: int, kind: int = H.SHOT_TRAINING, first: int = 0) -> List[S.Spec]:
    dt = surrogate_dt()
    return [draw_spec(seed, first + i, kind, dt) for i in range(n)]


def inputs_of(specs: List[S.Spec]):
    mats = np.stack([np.stack([sp.cell_vp, sp.cell_vs, sp.cell_rho], axis=-1).reshape(GRID, GRID, 3)
                     for sp in specs]).astype(np.float32)
    src = np.array([[sp.sources[0].x / CELL, sp.sources[0].y / CELL] for sp in specs], dtype=np.float32)
    return mats, src


def generate(seed: int, n: int, kind: int = H.SHOT_TRAINING, first: int = 0, chunk: int = 1000) -> Dataset:
    """Draws first..first+n-1 of (seed, kind) solved by the batched FP32 solver."""
    t0 = time.perf_counter()
    specs = specs_of(seed, n, kind, first)
    mats, src = inputs_of(specs)
    traces, secs = solve(specs, chunk=chunk)
    return Dataset(mats, src, traces, np.full(n, kind), secs, time.perf_counter() - t0, specs)


def concat(*ds: Dataset) -> Dataset:
    specs = sum([list(d.specs) for d in ds], []) if all(d.specs is not None for d in ds) else None
    return Dataset(np.concatenate([d.materials for d in ds]), np.concatenate([d.src for d in ds]),
                   np.concatenate([d.traces for d in ds]), np.concatenate([d.kind for d in ds]),
                   sum(d.seconds for d in ds), sum(d.wall_seconds for d in ds), specs)


# Coarser solvers for the comparison at equal misfit: (elements per side, degree).  Each
# runs the same draw on the same 4 km square with block-averaged cell materials, the same
# source, wavelet and receivers, and the largest time step r * dt (r = 1, 2 or 4) within
# 0.5 x its CFL step at Vp = 7500 m/s, so its samples fall on the same times.
LADDER = [(64, 4), (64, 3), (64, 2), (32, 4), (32, 3), (32, 2), (16, 4), (16, 2)]


def coarse_spec(sp: S.Spec, mx: int, p: int, dt: float):
    """(the draw on mx x mx elements of degree p, time-step ratio r)."""
    f = GRID // mx
    if f * mx != GRID:
        raise ValueError(f"{mx} does not divide {GRID}")

    def avg(a):
        return np.asarray(a, dtype=np.float64).reshape(mx, f, mx, f).mean(axis=(1, 3)).ravel()

    probe = S.Spec(mx=mx, my=mx, p=p, scale=(GRID * CELL, GRID * CELL), shift=(0.0, 0.0), vp=7500.0,
                   vs=7500.0 / 1.6, rho=2500.0, cfl=0.5, tmax=1.0e30, nt=1)
    dt_max = H.Setup(probe).dt
    r = max(k for k in (1, 2, 4) if k * dt <= dt_max * (1.0 + 1e-12))
    return sp.replace(mx=mx, my=mx, p=p, cell_vp=avg(sp.cell_vp), cell_vs=avg(sp.cell_vs), cell_rho=avg(sp.cell_rho),
                      dt=r * dt, nt=NSTEPS // r), r


def solver_ladder(specs: List[S.Spec], true: np.ndarray, ladder=LADDER, threads: int = 16) -> List[dict]:
    """Misfit against `true` (the draws' fine traces) and throughput of each coarser solver."""
    dt = specs[0].dt
    out = []
    for mx, p in ladder:
        t0 = time.perf_counter()
        cs = [coarse_spec(sp, mx, p, dt) for sp in specs]
        r = cs[0][1]
        tr, secs = solve([c for c, _ in cs], chunk=len(cs), threads=threads, nsteps=NSTEPS // r, decimate=DECIMATE // r)
        wall = time.perf_counter() - t0
        mis = rel_l2(tr, true)
        nodes = (p * mx + 1) ** 2
        out.append({"mx": mx, "p": p, "dt_ratio": r, "nodes": nodes, "solver_seconds": secs, "wall_seconds": wall,
                    "draws_per_s": len(specs) / wall, "misfit_mean": float(mis.mean()),
                    "misfit_median": float(np.median(mis)), "misfit_p90": float(np.percentile(mis, 90))})
    return out


def equal_misfit(ladder: List[dict], misfit: float, draws_per_s: float) -> dict:
    """The fastest ladder solver whose mean misfit is at most `misfit`, and the gain of a method of
    that misfit and throughput over it (None when no coarser solver is that accurate): `gain`
    against the solver's wall time (host set-up of the draws included), `gain_solver_time`
    against its device time alone."""
    ok = [e for e in ladder if e["misfit_mean"] <= misfit]
    if not ok:
        return {"solver": None, "gain": None, "gain_solver_time": None}
    best = max(ok, key=lambda e: e["draws_per_s"])
    n = best["draws_per_s"] * best["wall_seconds"]
    return {"solver": best, "gain": draws_per_s / best["draws_per_s"],
            "gain_solver_time": draws_per_s * best["solver_seconds"] / n}


def rel_l2(pred: np.ndarray, true: np.ndarray) -> np.ndarray:
    """Per-draw relative L2 misfit over all receivers, components and samples."""
    p = pred.reshape(pred.shape[0], -1).astype(np.float64)
    t = true.reshape(true.shape[0], -1).astype(np.float64)
    return np.linalg.norm(p - t, axis=1) / np.maximum(np.linalg.norm(t, axis=1), 1e-300)


def net_config(max_batch: int = 32) -> N.Config:
    """The 4-layer, width-64, 16-mode operator on the 128^2 cell grid; each receiver's column gives
    128 rows x 16 values = 2 components x 1024 samples (row k: samples 8k..8k+7)."""
    return N.Config(ny=GRID, nx=GRID, cin=16, width=64, modes=16, layers=4, nrec=NREC, nout=2 * NSAMP,
                    hidden=128, max_batch=max_batch)


SUB = DECIMATE * 2      # values per grid row and receiver: 2 components x 8 samples (rows = 1024 / 8)


def to_net_layout(traces: np.ndarray) -> np.ndarray:
    """[n, 16, 2 x 1024] traces -> the network's output layout [n, 16, 128 rows, 2 x 8]:
    row k of a receiver's column carries samples 8k..8k+7 of both components."""
    n = traces.shape[0]
    rows = NSAMP // 8
    return np.ascontiguousarray(traces.reshape(n, NREC, 2, rows, 8).transpose(0, 1, 3, 2, 4).reshape(n, NREC, -1))


def from_net_layout(out: np.ndarray) -> np.ndarray:
    n = out.shape[0]
    rows = NSAMP // 8
    return np.ascontiguousarray(out.reshape(n, NREC, rows, 2, 8).transpose(0, 1, 3, 2, 4).reshape(n, NREC, -1))


def mirrored(ds: Dataset) -> Dataset:
    """The draws mirrored in x: exact solutions of the mirrored problems.  The receivers sit
    symmetrically (x_r = L - x_{15-r}, on mirrored cells), so receiver r of the mirror is receiver
    15 - r of the original with vx negated."""
    tr = ds.traces.reshape(len(ds), NREC, 2, NSAMP)[:, ::-1].copy()
    tr[:, :, 0] *= -1.0
    src = ds.src.copy()
    src[:, 0] = GRID - src[:, 0]
    return Dataset(np.ascontiguousarray(ds.materials[:, :, ::-1, :]), src, tr.reshape(len(ds), NREC, -1),
                   ds.kind.copy(), 0.0, 0.0, None)


class DeviceData:
    """A data set resident on the GPU: materials, source cells and scaled targets (network layout)."""

    def __init__(self, ds: Dataset, scale: Optional[float] = None, augment: bool = False):
        import torch
        if augment:
            ds = concat(ds, mirrored(ds))
        self.n = len(ds)
        self.materials = torch.from_numpy(ds.materials).cuda()
        self.src = torch.from_numpy(ds.src).cuda()
        self.scale = float(np.sqrt(np.mean(ds.traces.astype(np.float64) ** 2))) if scale is None else scale
        self.targets = torch.from_numpy(to_net_layout(ds.traces / self.scale)).cuda()
        self.true = ds.traces


def train(data: DeviceData, idx_train: np.ndarray, rec_x: np.ndarray, seed: int = 0, epochs: int = 20,
          batch: int = 32, lr: float = 1e-3, lr_min: float = 1e-5, log=None):
    """Adam on the mean-squared error of the scaled traces, cosine learning-rate decay.
    Returns (network, {"loss": per-epoch mean, "samples_per_s": training throughput})."""
    import torch
    cfg = net_config(batch)
    net = N.Network(cfg, seed=seed)
    net.set_receivers(rec_x)
    stream = torch.cuda.Stream()
    net.set_stream(stream.cuda_stream)
    x = torch.zeros(batch, GRID, GRID, cfg.cin, dtype=torch.bfloat16, device="cuda")
    t = torch.zeros(batch, NREC, cfg.nout, device="cuda")
    rng = np.random.default_rng(seed + 7)
    steps_per_epoch = len(idx_train) // batch
    total = steps_per_epoch * epochs
    hist, step = [], 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for ep in range(epochs):
        perm = rng.permutation(idx_train)
        losses = []
        for s in range(steps_per_epoch):
            with torch.cuda.stream(stream):
                idx = torch.from_numpy(perm[s * batch:(s + 1) * batch].astype(np.int32)).cuda()
                net.build_inputs(data.materials, data.src, idx, SIGMA_CELLS, x)
                net.gather_targets(data.targets, idx, t)
            losses.append(net.loss_grad(x, t))
            cur = lr_min + 0.5 * (lr - lr_min) * (1.0 + np.cos(np.pi * step / max(1, total)))
            net.adam_step(float(cur), 0.9, 0.999, 1e-8, 0.0)
            step += 1
        hist.append(float(np.mean(losses)))
        if log:
            log(f"net {seed} epoch {ep} loss {hist[-1]:.4e}")
    ev1.record(stream)
    torch.cuda.synchronize()
    secs = ev0.elapsed_time(ev1) / 1e3
    return net, {"loss": hist, "samples_per_s": total * batch / secs, "seconds": secs, "steps": total}


def for_inference(nets, max_batch: int = 128, rec_x: Optional[np.ndarray] = None):
    """Copies of trained networks whose activation buffers take `max_batch` draws per
    forward pass (training runs 32): the small GEMMs of one pass are latency-bound, so
    larger passes serve more draws per second.  Parameters and receivers are the same."""
    out = []
    for net in nets:
        cfg = dataclasses.replace(net.cfg, max_batch=max_batch)
        n2 = N.Network(cfg, seed=0)
        n2.set_params(net.params())
        n2.set_receivers(net.rec_x if rec_x is None else rec_x)
        out.append(n2)
    return out


def predict(nets, data: DeviceData, idx: np.ndarray, batch: Optional[int] = None) -> np.ndarray:
    """[K, n, 16, 2048] predictions (unscaled) of every network for draws idx, `batch` draws per
    pass (default: what the networks' buffers take).  The outputs stay on the device until all
    batches are done, then come back in one copy."""
    import torch
    K = len(nets)
    if batch is None:
        batch = min(net.cfg.max_batch for net in nets)
    stream = torch.cuda.Stream()
    for net in nets:
        net.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        x = torch.zeros(batch, GRID, GRID, 16, dtype=torch.bfloat16, device="cuda")
        y = torch.zeros(K, len(idx), NREC, 2 * NSAMP, device="cuda")
        it_all = torch.from_numpy(np.ascontiguousarray(idx, dtype=np.int32)).cuda()
        for b0 in range(0, len(idx), batch):
            n = min(batch, len(idx) - b0)
            nets[0].build_inputs(data.materials, data.src, it_all[b0:b0 + n], SIGMA_CELLS, x[:n])
            for k, net in enumerate(nets):
                net.forward(x[:n], y[k, b0:b0 + n])
        yk = y.cpu().numpy()
    out = np.empty((K, len(idx), NREC, 2 * NSAMP), dtype=np.float32)
    for k in range(K):
        out[k] = from_net_layout(yk[k]) * np.float32(data.scale)
    return out


def disagreement(preds: np.ndarray) -> np.ndarray:
    """Ensemble-disagreement estimate per draw: mean over members of ||p_k - mean|| / ||mean||
    (infinite with fewer than two members: nothing can be accepted)."""
    if preds.shape[0] < 2:
        return np.full(preds.shape[1], np.inf)
    mean = preds.mean(axis=0)
    num = np.linalg.norm((preds - mean[None]).reshape(preds.shape[0], preds.shape[1], -1), axis=2).mean(axis=0)
    den = np.maximum(np.linalg.norm(mean.reshape(mean.shape[0], -1), axis=1), 1e-300)
    return num / den


def serve(nets, data: DeviceData, specs: List[S.Spec], threshold: float = 0.01, audit: float = 0.05,
          batch_requests: int = 1000, seed: int = 0) -> dict:
    """Serve draws in batches: the ensemble's mean prediction is returned when its disagreement is
    <= threshold, otherwise the batched FP32 solver recomputes the draw; a random `audit` fraction of
    the accepted draws is re-solved as well to measure the accepted misfit.  Latency of a request =
    from its batch's arrival to its result."""
    rng = np.random.default_rng(seed)
    n = data.n
    lat = np.zeros(n)
    acc_all = np.zeros(n, dtype=bool)
    result = np.zeros_like(data.true)
    audit_mis = []
    t_start = time.perf_counter()
    t_sur_total = 0.0
    for q0 in range(0, n, batch_requests):
        q = np.arange(q0, min(n, q0 + batch_requests))
        t0 = time.perf_counter()
        preds = predict(nets, data, q)
        mean, dis = preds.mean(axis=0), disagreement(preds)
        t_sur = time.perf_counter() - t0
        t_sur_total += t_sur
        acc = dis <= threshold
        aud = acc & (rng.random(len(q)) < audit)
        need = np.where(~acc | aud)[0]
        solved = solve([specs[q[i]] for i in need], chunk=max(1, len(need)))[0] if len(need) else None
        t_done = time.perf_counter() - t0
        result[q[acc]] = mean[acc]
        if solved is not None:
            pos = {int(i): k for k, i in enumerate(need)}
            rej = np.where(~acc)[0]
            if len(rej):
                result[q[rej]] = solved[[pos[int(i)] for i in rej]]
            au = np.where(aud)[0]
            if len(au):
                audit_mis.extend(rel_l2(mean[au], solved[[pos[int(i)] for i in au]]).tolist())
        lat[q[acc]] = t_sur
        lat[q[~acc]] = t_done
        acc_all[q] = acc
    total = time.perf_counter() - t_start
    true_mis = rel_l2(result, data.true)
    return {"requests": n, "threshold": threshold, "seconds": total, "seismograms_per_s": n / total,
            "fallback_rate": float(1.0 - acc_all.mean()), "accepted": int(acc_all.sum()),
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "surrogate_seconds": t_sur_total,
            "audit": {"n": len(audit_mis), "mean_misfit": float(np.mean(audit_mis)) if audit_mis else None,
                      "max_misfit": float(np.max(audit_mis)) if audit_mis else None},
            "served_misfit": {"mean": float(true_mis.mean()), "p99": float(np.percentile(true_mis, 99)),
                              "max": float(true_mis.max())}}


def forward_flops(cfg: N.Config) -> float:
    """Tensor-core FLOPs of one sample's forward pass (2 M N K summed over the GEMMs)."""
    ny, nx, w, m, L = cfg.ny, cfg.nx, cfg.width, cfg.modes, cfg.layers
    npix = ny * nx
    f = 2.0 * npix * cfg.cin * w                                   # lift
    per_layer = (2.0 * ny * (2 * m) * w * nx                       # DFT along x
                 + 2.0 * (4 * m) * (m * w) * (2 * ny)              # DFT along y
                 + 2.0 * (2 * m * m) * (2 * w) * (2 * w)           # mode mixing
                 + 2.0 * (2 * ny) * (m * w) * (4 * m)              # inverse along y
                 + 2.0 * ny * nx * w * (2 * m)                     # inverse along x
                 + 2.0 * npix * w * w)                             # 1x1 convolution
    f += L * per_layer
    f += 2.0 * cfg.nrec * ny * (w * cfg.hidden + cfg.hidden * (cfg.nout // ny))
    return f
