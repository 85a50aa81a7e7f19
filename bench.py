"""Benchmark of the GB300 SEM time loop: DOF-updates/s.

Default workload: the 2048 x 2048-element, degree-4 heterogeneous solve (20 km
square, Gaussian-random-field Vp, 64 receivers; 67.1M GLL nodes, 134.3M DOF),
one GPU, FP32 with Kahan-compensated updates as the headline, FP64 (reference
operation order) measured beside it.  A "step" is one explicit time step of the
whole mesh (the loop body of se2wave.c:4722-4775).  The state (5.4 GB in FP32+
Kahan, 6.4 GB in FP64) is far larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores (the oracle
port, bit-identical to se2wave.c compiled in place) on a bounded sample of the
same workload, one independent solve per host thread.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF-updates/s"
ALG_BYTES_NOTE = "per node-step: read+write of the fields, lumped mass, cell Lame pair"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# DRAM bytes per node and step of the step kernels as ncu measured them (dram__bytes_read.sum +
# dram__bytes_write.sum of one launch at 1024^2, degree 4, divided by its 16.79M nodes; the
# kernel's traffic grows in proportion to the nodes, so it is scaled to the workload's node
# count), from the ncu capture of the persistent FP32+Kahan step kernel at 1024^2 (tile
# configuration 1: 7 x 7 elements, 320 threads, two owned buffers): 639.2 MB read + 493.6 MB written
MEASURED_TRAFFIC_PER_NODE = {"fp32_kahan": 1132.8e6 / 16785409}


def alg_bytes_per_node(precision: str, ne: int, nnodes: int) -> float:
    """Algorithmic DRAM bytes per node per step (unique traffic only)."""
    cell = ne / nnodes
    if precision == "fp64":
        return 2 * 3 * 16 + 8 + 16 * cell          # u,v,a (double2) in+out, M, (lambda, mu)
    # the plain and Kahan kernels read a float4 of constants per cell (lambda detJ, mu detJ,
    # d xi/dx, d eta/dy); the two-float kernel reads (lambda, mu) with their low parts
    if precision == "fp32_kahan":
        return 2 * 4 * 8 + 4 + 16 * cell           # leapfrog u,w,cu,cw (float2) in+out, 1/M, cell constants
    if precision == "fp32_df":
        return 2 * 4 * 8 + 8 + 16 * cell           # the same state, 1/M and (lambda, mu) with their low parts
    return 2 * 2 * 8 + 4 + 16 * cell               # leapfrog u,w (float2) in+out, 1/M, cell constants


def fp64_ops_per_node(p: int) -> float:
    """Algorithmic FP64 operations per node and step of the reference's arithmetic
    (se2wave.c:1321-1417 and 4724-4745) with its dense element sums restricted to the
    terms that are not exact zeros (the row and column of each point), as the FP64 kernel
    evaluates them, and without any halo recompute.  Per GLL point: strains 2 x N1 + 2 x N1
    + 4 x N1 (the shear sum over row and column with the diagonal term) multiplies and
    adds, c11 and the three stresses 9 -> 8 N1 + 9.  Per element node: the weak divergence
    over the 2 N1 - 1 points of its row and column, x and y: 6 per off-diagonal point and
    10 at the node itself -> 12 N1 - 2.  Per node: the element sums (N1^2 / p^2
    contributions per component), the three AXPYs of the predictor (12), f + g (4), a = f / M
    (2 divisions) and the corrector (4)."""
    n1 = p + 1
    per_element = n1 * n1 * (8 * n1 + 9) + n1 * n1 * (12 * n1 - 2)
    return per_element / (p * p) + 2.0 * n1 * n1 / (p * p) + 12 + 4 + 2 + 4


def df_ops_per_node(p: int) -> float:
    """Algorithmic FP32 arithmetic instructions per node and step of the two-float mode (no
    halo recompute): per (element, line) item, the displacement differences (TwoSum + 2,
    x and y: 16 p per direction), the derivative contractions as compensated dot products
    (12 per term, N1 p terms per component and direction) with one TwoSum normalisation per
    output (6), the Hooke stress and factors (145 per point, 29 per item), the xi and eta
    divergences (24 N1^2 + 12 N1 each); per node the element sum (11 per extra
    contribution and component), a = f / M (14) and the two updates (36 each)."""
    n1 = p + 1
    grad = 2 * (16 * p + 24 * p * n1 + 12 * n1)
    stress = 145 * n1 + 29
    div = 2 * (24 * n1 * n1 + 12 * n1)
    per_element = n1 * (grad + stress + div)
    extra = 2.0 * (n1 * n1 / (p * p) - 1.0) * 11
    return per_element / (p * p) + extra + 14 + 36 + 36


def reference_bytes_per_node(precision: str, ne: int, nnodes: int) -> float:
    """DRAM bytes per node per step of the reference's own update sequence (se2wave.c:4722-4775)
    in this precision: u, v, a read and written (FP32+Kahan: also the compensation terms of u
    and v), 1/M and the cell's (lambda, mu).  The kick-drift state above needs no a, so it moves
    fewer bytes for the same DOF-updates; this count is the one to compare other
    implementations of the reference's scheme against."""
    words = {"fp64": 13, "fp32": 13, "fp32_kahan": 21, "fp32_df": 22}[precision]   # two-float: 1/M's low part
    cell_words = 4 if precision == "fp32_df" else 2
    wb = 8 if precision == "fp64" else 4
    return (words + cell_words * ne / nnodes) * wb


def reference_formulation(precision: str, ne: int, nnodes: int, per_step: float, hbm: float) -> dict:
    rb = reference_bytes_per_node(precision, ne, nnodes)
    ach = rb * nnodes / per_step / 1e9
    return {"bytes_per_node": rb, "achieved": ach, "frac": ach / hbm,
            "note": "reference update sequence's bytes (u, v, a and Kahan terms of u, v) at the same step time"}


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(threads: int, rows: int, steps: int, warmup: int = 1, record: bool = True):
    """The oracle port (the reference algorithm) on host threads: each thread an
    independent solve of a 2048 x `rows` element strip of the workload, with receiver
    output (the reference's default) or without it (-ignore_receiver_output)."""
    from oracle import oracle as O
    from se2dr_fork_gb300 import spec as S
    from se2dr_fork_gb300 import host as H
    vp = H.gaussian_random_field(2048, rows, 5000.0, 0.1, 8.0, seed=2048)
    sp = S.grf2048(2048, rows, nt=warmup + steps + 2, cells=(vp, vp / 1.73, np.full_like(vp, 2700.0)))
    # same element shape as the full workload: the strip is rows/2048 of its height
    h = 20000.0 * rows / 2048.0
    sp = sp.replace(scale=(20000.0, h), shift=(-10000.0, -h / 2), receivers=[(x, 0.0) for x, _ in sp.receivers])
    secs = O.bench(sp, threads, warmup, steps, record=record)
    dof = sp.ndof
    rec = "receivers recorded" if record else "-ignore_receiver_output"
    return {"value": threads * dof * steps / secs, "seconds": secs, "dof_per_thread": dof,
            "sample": f"{threads} independent solves of a 2048x{rows}-element strip of the workload "
                      f"(degree 4, {dof} DOF each, {rec}), {steps} steps after {warmup} warm-up"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # calibrate the strip so the whole run stays within ~3 minutes
    probe = cpu_baseline(threads, 8, 1, 0)
    per_row = probe["seconds"] / 8.0
    budget = 150.0 / max(1, args.steps + args.warmup)
    rows = int(max(1, min(64, budget / max(per_row, 1e-6))))
    res = cpu_baseline(threads, rows, args.steps, args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": "DOF/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * res["seconds"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "grf2048: 2048x2048 elements, degree 4, 20 km square, GRF Vp, 64 receivers",
                       "sample": res["sample"], "host_threads": threads},
            "cpu_baseline": {"value": res["value"], "unit": "DOF/s", "cores": threads, "kind": "port",
                             "sample": res["sample"]},
            "e2e": {"value": res["value"], "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def replica_seconds(local_seconds: float, dist=None, device=None) -> float:
    """Job time of N independent replicas: the slowest rank (max over ranks)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return local_seconds
    import torch
    t = torch.tensor([local_seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_sum(x: float, dist=None, device: str = "cpu") -> float:
    """Sum of a per-rank quantity over all ranks (the work of ranks that ran different shots)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def replica_value(dof_per_replica: int, steps: int, world: int, seconds: float) -> float:
    """Whole-job DOF-updates/s of `world` replicas of the same workload (weak scaling)."""
    return world * dof_per_replica * steps / seconds


def median_job(runs):
    """The median of end-to-end jobs [(seconds, parts)]: the (seconds, parts) of the middle
    one by time (the upper middle for an even count)."""
    return sorted(runs, key=lambda r: r[0])[len(runs) // 2]


def time_steps(sol, steps, warmup, stream, torch):
    """Device time of `steps` steps (CUDA events on the launching stream)."""
    sol.advance(warmup)
    sol.traces()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    launches0 = sol.info()["launches"]
    torch.cuda.synchronize()
    ev0.record(stream)
    sol.advance(steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = sol.info()["launches"] - launches0
    sol.traces()
    return ev0.elapsed_time(ev1) / 1e3, launches


def run_ours(args, rank, world):
    import torch
    from se2dr_fork_gb300 import gpu as G
    from se2dr_fork_gb300 import host as H
    from se2dr_fork_gb300 import spec as S

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def tmax(x):
        return replica_seconds(x, dist, "cuda")

    spec = S.grf2048(args.mx, args.mx, p=args.degree, nt=args.steps + args.warmup + 10)
    setup = H.Setup(spec)
    nnodes, ne = setup.nnodes, setup.mx * setup.my
    dof = 2 * nnodes
    stream = torch.cuda.Stream()
    hbm, peak_kind = peaks()
    results = {}
    from se2dr_fork_gb300 import autotune
    tuned = None
    if args.autotune and args.precision != "fp64":
        tuned = autotune.tune(setup, args.precision, steps=10)
    legs = [args.precision] + (["fp64"] if args.precision != "fp64" and not args.no_fp64 else [])
    if args.precision != "fp32_df" and not args.no_df:
        legs.append("fp32_df")
    pipe = {}
    for kind in ("fp64_mul_add", "fp32_mul_add"):
        try:
            pipe[kind] = G.pipe_peak(kind)
        except Exception:
            pipe[kind] = None
    for prec in legs:
        k = args.steps if prec == args.precision else max(3, args.steps // (8 if prec == "fp64" else 2))
        sol = G.Solver(setup, prec, trace_capacity=k + args.warmup + 2)
        if prec != "fp64":
            if args.tile_config >= 0:
                sol.set_tile_config(args.tile_config)
            else:
                autotune.apply(sol, prec)
        sol.set_stream(stream.cuda_stream)
        barrier()
        with ClockSampler(local) as clk:
            secs, launches = time_steps(sol, k, args.warmup, stream, torch)
        secs = tmax(secs)
        tile = sol.tile_config_info(sol.tile_config) if prec != "fp64" else None
        sol.close()
        per = secs / k
        b = alg_bytes_per_node(prec, ne, nnodes)
        achieved = b * nnodes / per / 1e9
        results[prec] = {"value": replica_value(dof, k, world, secs), "ms_per_step": 1e3 * per, "steps": k, "tile": tile,
                         "launches": launches, "clocks": clk.summary(),
                         "roofline": {"bound": "hbm" if prec != "fp64" else "fp64 pipe (HBM fraction shown)",
                                      "achieved": achieved, "peak": hbm, "unit": "GB/s",
                                      "frac": achieved / hbm,
                                      "traffic": (MEASURED_TRAFFIC_PER_NODE[prec] * nnodes
                                                  if prec in MEASURED_TRAFFIC_PER_NODE and args.mx == 2048
                                                  and args.degree == 4 else None),
                                      "traffic_note": "ncu DRAM bytes per node at 1024^2 x nodes (bytes per launch)",
                                      "alg_bytes_per_node": b, "peak_kind": peak_kind,
                                      "reference_formulation": reference_formulation(prec, ne, nnodes, per, hbm)}}
        # the arithmetic roof of the kernels that HBM does not bound, against the pipe rate
        # measured on this device (se2gpu_pipe_peak)
        ops, kind = {"fp64": (fp64_ops_per_node, "fp64_mul_add"), "fp32_df": (df_ops_per_node, "fp32_mul_add")}.get(
            prec, (None, None))
        if ops and pipe.get(kind):
            ach = ops(args.degree) * nnodes / per / 1e12
            results[prec]["pipe_roofline"] = {
                "bound": "fp64 pipe" if prec == "fp64" else "fp32 pipe", "achieved": ach, "peak": pipe[kind] / 1e12,
                "unit": "Tops/s", "frac": ach / (pipe[kind] / 1e12), "ops_per_node": ops(args.degree),
                "peak_kind": "measured (se2gpu_pipe_peak %s)" % kind,
                "note": "algorithmic arithmetic operations per node (no halo recompute) x nodes / step time"}

    # end to end through the C-ABI: create (upload from host) + K steps + traces read back +
    # destroy, three times (each a complete job); the median job is reported, every run listed
    prec = args.precision
    runs = []
    for _ in range(3):
        barrier()
        t0 = time.perf_counter()
        sol = G.Solver(setup, prec, trace_capacity=args.steps + 2)
        if prec != "fp64":
            if args.tile_config >= 0:
                sol.set_tile_config(args.tile_config)
            else:
                autotune.apply(sol, prec)
        t_create = time.perf_counter()
        sol.advance(args.steps)
        tr = sol.traces()
        t_steps = time.perf_counter()
        sol.close()
        torch.cuda.synchronize()
        t_end = time.perf_counter()
        runs.append((tmax(t_end - t0), {"create_s": t_create - t0, "steps_and_traces_s": t_steps - t_create,
                                        "destroy_s": t_end - t_steps}))
    e2e_s, e2e_parts = median_job(runs)
    e2e_runs = [r[0] for r in runs]
    # bytes of the caller's FP64 host arrays that se2gpu_create and advance read: the mass, the
    # cell Lame parameters, the Jacobians, D and the weights, the source values, the receiver
    # indices and the STF values of every step (the FP32 modes convert on the device)
    h2d = (nnodes * 8 + 2 * ne * 8 + 4 * (setup.mx + setup.my) * 8 + 2 * setup.npe * 16
           + setup.nsrc * 2 * setup.npe * 8 + 12 * setup.nrec + 8 * setup.nsrc * args.steps)
    d2h = tr.shape[0] * 7 * setup.nrec * 8

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    head = results[args.precision]
    cpu = None
    if world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        c = cpu_baseline(threads, args.cpu_rows, args.cpu_steps)
        cpu = {"value": c["value"], "unit": "DOF/s", "cores": threads, "kind": "port", "sample": c["sample"]}
        try:
            c1 = cpu_baseline(1, args.cpu_rows, max(2, args.cpu_steps // 2))
            cpu["single_core_value"] = c1["value"]
            cn = cpu_baseline(threads, args.cpu_rows, args.cpu_steps, record=False)
            cpu["no_receiver_output_value"] = cn["value"]
        except Exception:
            pass
    line = {"metric": METRIC, "value": head["value"], "unit": "DOF/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if prec != "fp64" else "f64", "data": "synthetic",
            "config": {"workload": f"grf2048: {args.mx}x{args.mx} elements, degree {args.degree}, 20 km square, "
                                   f"Gaussian-random-field Vp (mean 5000, 10% std, corr 8 cells), Vp/Vs 1.73, "
                                   f"rho 2700, explosive Ricker f0 8 Hz, 64 receivers",
                       "precision": prec, "nodes": nnodes, "dof": dof, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (state %.1f GB)" % ({"fp32_kahan": 8, "fp32_df": 8, "fp32": 4, "fp64": 6}[prec]
                                                                       * nnodes * (4 if prec != 'fp64' else 8) * 2 / 1e9)},
            "roofline": head["roofline"], "clocks": head["clocks"], "gpu_launches": head["launches"],
            "tile": head.get("tile"), "autotune": tuned,
            "e2e": {"value": world * dof * args.steps / e2e_s, "unit": "DOF/s", "h2d_bytes_per_step": h2d / args.steps,
                    "d2h_bytes_per_step": d2h / args.steps, "seconds": e2e_s, "parts": e2e_parts,
                    "runs_s": e2e_runs, "of_runs": "median of 3 complete jobs",
                    "includes": "se2gpu_create (upload of the set-up from host memory), advance, traces, destroy"},
            "cpu_baseline": cpu}
    for leg in ("fp64", "fp32_df"):
        if leg in results and args.precision != leg:
            r = results[leg]
            line[leg] = {"value": r["value"], "ms_per_step": r["ms_per_step"], "steps": r["steps"],
                         "roofline": r["roofline"], "pipe_roofline": r.get("pipe_roofline"), "clocks": r["clocks"]}
    if "pipe_roofline" in head:
        line["pipe_roofline"] = head["pipe_roofline"]
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_sweep(args):
    """Degree sweep at ~16M nodes: mx = 4000, 2000, 1333, 1000, 800, 667, 571, 500 for p = 1..8
    (GRF material as the 2048^2 workload, one JSON line per degree and precision)."""
    import torch
    from se2dr_fork_gb300 import autotune
    from se2dr_fork_gb300 import gpu as G
    from se2dr_fork_gb300 import host as H
    from se2dr_fork_gb300 import spec as S
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    hbm, _ = peaks()
    for p, mx in zip(range(1, 9), [4000, 2000, 1333, 1000, 800, 667, 571, 500]):
        vp = H.gaussian_random_field(mx, mx, 5000.0, 0.1, 8.0, seed=2048)
        sp = S.grf2048(mx, mx, p=p, nt=10 ** 6, cells=(vp, vp / 1.73, np.full_like(vp, 2700.0)))
        setup = H.Setup(sp)
        for prec in ["fp32_kahan", "fp64"]:
            k = args.steps if prec != "fp64" else max(3, args.steps // 10)
            if prec != "fp64" and args.autotune:
                autotune.tune(setup, prec, steps=5)
            sol = G.Solver(setup, prec, trace_capacity=k + args.warmup + 2)
            if prec != "fp64":
                autotune.apply(sol, prec)
            sol.set_stream(stream.cuda_stream)
            secs, launches = time_steps(sol, k, args.warmup, stream, torch)
            tile = sol.tile_config_info(sol.tile_config) if prec != "fp64" else None
            sol.close()
            per = secs / k
            b = alg_bytes_per_node(prec, setup.mx * setup.my, setup.nnodes)
            print(json.dumps({"sweep": "degree", "p": p, "mx": mx, "nodes": setup.nnodes, "precision": prec,
                              "dof_updates_per_s": 2 * setup.nnodes * k / secs, "ms_per_step": 1e3 * per,
                              "hbm_frac": b * setup.nnodes / per / 1e9 / hbm, "tile": tile, "steps": k}), flush=True)
        del setup


def trace_errors(tr, ref, k):
    """Relative L2 of each receiver trace component (ux uy vx vy ax ay) against `ref`, and of
    curl(v) on the scale k |v| of the velocity gradient (an explosive source's curl is
    discretisation noise, so its own norm measures nothing)."""
    errs = []
    for c in range(6):
        den = np.linalg.norm(ref[:, 1 + c::7])
        errs.append(float(np.linalg.norm(tr[:, 1 + c::7] - ref[:, 1 + c::7]) / (den if den > 0 else 1.0)))
    vn = np.sqrt(np.linalg.norm(ref[:, 3::7]) ** 2 + np.linalg.norm(ref[:, 4::7]) ** 2)
    scale = max(np.linalg.norm(ref[:, 7::7]), k * vn)
    errs.append(float(np.linalg.norm(tr[:, 7::7] - ref[:, 7::7]) / (scale if scale > 0 else 1.0)))
    return errs


def run_accuracy(args):
    """FP32 modes against FP64 on the same problem over --steps steps: relative L2 of every
    receiver trace component and of the final u, v, a fields, one JSON line per precision.
    The 2048^2 degree-4 workload (64 receivers on y = 2500 m; its default 20000 steps reach
    t = 1.04 s, past the P and S arrivals), or with --sweep the degree-sweep meshes."""
    import torch
    from se2dr_fork_gb300 import gpu as G
    from se2dr_fork_gb300 import host as H
    from se2dr_fork_gb300 import spec as S
    torch.cuda.set_device(0)
    cases = list(zip(range(1, 9), [4000, 2000, 1333, 1000, 800, 667, 571, 500])) if args.sweep else [(args.degree, args.mx)]
    k_shear = 2.0 * np.pi * 8.0 / (5000.0 / 1.73)   # Ricker f0 over the mean shear speed
    for p, mx in cases:
        vp = H.gaussian_random_field(mx, mx, 5000.0, 0.1, 8.0, seed=2048)
        cells = (vp, vp / 1.73, np.full_like(vp, 2700.0))
        steps = args.steps
        if args.acc_tmax > 0:   # as many steps as reach this time on this mesh
            steps = int(np.ceil(args.acc_tmax / H.Setup(S.grf2048(mx, mx, p=p, nt=1, cells=cells)).dt))
        setup = H.Setup(S.grf2048(mx, mx, p=p, nt=steps, cells=cells))
        ref = None
        for prec in ["fp64", "fp32_df", "fp32_kahan", "fp32"]:
            sol = G.Solver(setup, prec, trace_capacity=min(steps, 2000))
            t0 = time.time()
            tr = sol.run(steps, block=2000)
            sol.synchronize()
            secs = time.time() - t0
            fields = sol.fields()
            sol.close()
            if prec == "fp64":
                ref = (tr, fields)
                errs, ferr = None, None
            else:
                errs = trace_errors(tr, ref[0], k_shear)
                ferr = {n: float(np.linalg.norm(x - y) / np.linalg.norm(y)) for n, x, y in zip("uva", fields, ref[1])}
            print(json.dumps({"accuracy": "sweep" if args.sweep else "grf2048", "p": p, "mx": mx, "nodes": setup.nnodes,
                              "steps": steps, "t_end": float(tr[-1, 0]) if len(tr) else 0.0,
                              "receivers": setup.nrec, "precision": prec, "wall_s": secs,
                              "trace_rel_l2": dict(zip(["ux", "uy", "vx", "vy", "ax", "ay", "curl"], errs)) if errs else None,
                              "field_rel_l2": ferr}), flush=True)
            del fields
        del setup, ref


def run_ensemble(args, rank: int = 0, world: int = 1):
    """Batched ensemble: `--shots` seeded shots (mx, my ~ U{32..512}, p in {3,4,6}, 2 layers +
    elliptical inclusion, random source and moment tensor, Ricker f0 ~ U[5,20] Hz, 32 receivers,
    5000 steps each), FP32 with Kahan-compensated updates, one persistent launch per degree group
    per step, blocks of steps replayed as CUDA graphs.  Prints one JSON line."""
    import concurrent.futures as cf
    import torch
    from se2dr_fork_gb300 import gpu as G
    from se2dr_fork_gb300 import host as H
    from se2dr_fork_gb300 import spec as S
    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:   # one block of shots per GPU, no collective on the data path (timing only)
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    t0 = time.perf_counter()
    specs = S.ensemble_shard(args.shots, rank, seed=3)
    if args.ens_degree > 0:   # the same shots, all at one degree (per-degree efficiency of the batch kernel)
        specs = [sp.replace(p=args.ens_degree) for sp in specs]
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        setups = list(ex.map(H.Setup, specs))
    t_setup = time.perf_counter() - t0
    prec = args.precision if args.precision != "fp64" else "fp32_kahan"
    t0 = time.perf_counter()
    ens = G.Ensemble(setups, prec, block=args.block)
    t_create = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    ens.set_stream(stream.cuda_stream)
    nodes = sum(su.nnodes for su in setups)
    ne = sum(su.mx * su.my for su in setups)
    dof = 2 * nodes
    hbm, peak_kind = peaks()
    b = alg_bytes_per_node(prec, ne, nodes)

    def timed(nsteps):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        ens.enqueue(nsteps)
        ev1.record(stream)
        torch.cuda.synchronize()
        ens.synchronize()
        return ev0.elapsed_time(ev1) / 1e3

    tuned = {}
    if args.autotune:
        for p in ens.degrees():
            times = []
            for c in range(8):
                try:
                    ens.set_tile_config(p, c)
                except G.GpuError:
                    break
                timed(args.block)
                times.append(timed(args.block))
            best = int(np.argmin(times))
            ens.set_tile_config(p, best)
            tuned[p] = {"config": best, "seconds": times}
    ens.advance(args.block, traces=False)          # stage real STF values, build the graphs
    timed(args.warmup * args.block)
    launches0 = ens.info()["launches"]
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        secs = timed(args.steps)
    launches = ens.info()["launches"] - launches0
    secs = replica_seconds(secs, dist, "cuda")
    dof_job = job_sum(dof, dist, "cuda")
    per = secs / args.steps
    achieved = b * nodes / per / 1e9
    # end to end through the C-ABI: host STF upload per block, receiver rows back to host memory
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    trs = ens.advance(args.steps)
    e2e_s = replica_seconds(time.perf_counter() - t0, dist, "cuda")
    nrec_total = sum(su.nrec for su in setups)
    nsrc_total = sum(su.nsrc for su in setups)
    steps_per_shot = 5000
    if rank != 0:
        ens.close()
        dist.destroy_process_group()
        return
    line = {"metric": METRIC, "value": dof_job * args.steps / secs, "unit": "DOF/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup * args.block, "ms_per_step": 1e3 * per, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"ensemble: {args.shots} shots, mx, my ~ U{{32..512}}, p in {{3,4,6}}, 2 layers + "
                                   f"elliptical inclusion, random moment tensor, Ricker f0 ~ U[5,20] Hz, 32 receivers",
                       "precision": prec, "nodes": nodes, "dof": dof, "block": args.block,
                       "parallelism": f"shot shards x{world} ({args.shots} shots per GPU)",
                       "degrees": {str(p): sum(1 for su in setups if su.p == p) for p in ens.degrees()},
                       "tile_configs": {str(p): ens.tile_config(p) for p in ens.degrees()},
                       "l2": "inputs larger than L2 (state %.1f GB)" % (nodes * 8 * (4 if prec == "fp32_kahan" else 2) / 1e9)},
            "shots_per_s": world * args.shots * (args.steps / secs) / steps_per_shot,
            "shot_steps": steps_per_shot,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": None, "alg_bytes_per_node": b, "peak_kind": peak_kind,
                         "reference_formulation": reference_formulation(prec, ne, nodes, per, hbm)},
            "clocks": clk.summary(), "gpu_launches": launches, "autotune": tuned or None,
            "e2e": {"value": dof_job * args.steps / e2e_s, "unit": "DOF/s", "seconds": e2e_s,
                    "shots_per_s": world * args.shots * (args.steps / e2e_s) / steps_per_shot,
                    "h2d_bytes_per_step": 8 * nsrc_total, "d2h_bytes_per_step": 8 * 7 * nrec_total,
                    "includes": "se2gpu_ensemble_advance: host STF upload per block, receiver rows to host memory"},
            "setup_seconds": {"host": t_setup, "ensemble_create": t_create},
            "trace_rows": int(sum(t.shape[0] for t in trs))}
    ens.close()
    if dist:
        dist.destroy_process_group()
    print(json.dumps(line), flush=True)


def run_surrogate(args):
    """Surrogate workload: training data from the batched FP32 solver, an ensemble of networks trained
    with the project's BF16 kernels, held-out misfit, and serving with the disagreement gate + solver
    fallback against the plain batched solver on the same draws.  Prints one JSON line."""
    import torch
    from se2dr_fork_gb300 import host as H
    from se2dr_fork_gb300 import surrogate as SU
    torch.cuda.set_device(0)
    log = (lambda m: print(m, file=sys.stderr, flush=True))
    t0 = time.perf_counter()
    tr = SU.generate(4, args.train, H.SHOT_TRAINING)
    log(f"training data: {args.train} draws in {tr.wall_seconds:.1f} s (solver {tr.seconds:.1f} s)")
    nood = max(1, int(round(0.1 * args.test)))
    te_in = SU.generate(5, args.test, H.SHOT_TRAINING)
    te_ood = SU.generate(6, nood, H.SHOT_OOD)
    test = SU.concat(te_in, te_ood)
    t_data = time.perf_counter() - t0
    dtrain = SU.DeviceData(tr, augment=True)
    dtest = SU.DeviceData(test, scale=dtrain.scale)
    rec_x = SU.receiver_cells(tr.specs[0])
    nets, stats = [], []
    for k in range(args.members):
        net, st = SU.train(dtrain, np.arange(dtrain.n), rec_x, seed=k, epochs=args.epochs, batch=32, lr=args.lr,
                           log=log)
        nets.append(net)
        stats.append(st)
    fwd = SU.forward_flops(SU.net_config())
    inf = SU.for_inference(nets, 128)   # the same networks, 128 draws per forward pass
    # inference throughput of the ensemble of networks, warm (a first call on a few draws
    # builds the streams and buffers), host-timed including the copy back
    SU.predict(inf, dtest, np.arange(min(dtest.n, 64)))
    torch.cuda.synchronize()
    tq = time.perf_counter()
    preds = SU.predict(inf, dtest, np.arange(dtest.n))
    t_pred = time.perf_counter() - tq
    mean, dis = preds.mean(axis=0), SU.disagreement(preds)
    mis = SU.rel_l2(mean, test.traces)
    is_ood = test.kind == H.SHOT_OOD
    what_if = []
    for th in (0.01, 0.02, 0.05, 0.1, 0.2, 0.5):
        acc = dis <= th
        what_if.append({"threshold": th, "fallback_rate": float(1 - acc.mean()),
                        "accepted_misfit_max": float(mis[acc].max()) if acc.any() else None,
                        "accepted_misfit_mean": float(mis[acc].mean()) if acc.any() else None})
    served = SU.serve(inf, dtest, test.specs, threshold=args.threshold, audit=0.05, batch_requests=args.serve_batch)
    solver_sps = dtest.n / test.wall_seconds
    # the gain at equal misfit: coarser solvers on (the first --ladder-draws of) the
    # in-distribution held-out draws, against the network's misfit on the same draws
    nl = min(len(te_in), args.ladder_draws)
    ladder = SU.solver_ladder(te_in.specs[:nl], te_in.traces[:nl])
    sur_sps = dtest.n / t_pred
    eq = SU.equal_misfit(ladder, float(mis[:nl].mean()), sur_sps)
    log(f"equal misfit: {eq}")
    line = {"metric": "seismograms/s surrogate vs solver @1% L2", "value": served["seismograms_per_s"],
            "unit": "seismograms/s", "n_gpus": 1, "higher_is_better": True, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": f"{args.train} training draws, {args.test} held-out + {nood} out-of-distribution "
                                   "requests; 128x128 elements, degree 4, 4096 steps, 16 receivers x 2 x 1024",
                       "network": "4 Fourier layers, width 64, 16 modes; column decoder 64-128-16 (GELU)",
                       "augmentation": "mirror in x (exact)", "members": args.members,
                       "epochs": args.epochs, "batch": 32},
            "solver_seismograms_per_s": solver_sps,
            "speedup_vs_solver": served["seismograms_per_s"] / solver_sps,
            "serving": served,
            "held_out": {"misfit_mean": float(mis[~is_ood].mean()), "misfit_median": float(np.median(mis[~is_ood])),
                         "misfit_p90": float(np.percentile(mis[~is_ood], 90)),
                         "ood_misfit_mean": float(mis[is_ood].mean()),
                         "disagreement_mean": float(dis[~is_ood].mean()), "ood_disagreement_mean": float(dis[is_ood].mean()),
                         "corr_disagreement_misfit": float(np.corrcoef(dis, mis)[0, 1])},
            "what_if": what_if,
            "equal_misfit": {"draws": nl, "surrogate_misfit_mean": float(mis[:nl].mean()),
                             "surrogate_draws_per_s": sur_sps, "fine_solver_draws_per_s": solver_sps,
                             "solver_ladder": ladder, "solver_at_equal_misfit": eq["solver"],
                             "gain_at_equal_misfit": eq["gain"],
                             "gain_at_equal_misfit_solver_device_time": eq["gain_solver_time"]},
            "training": {"samples_per_s": [st["samples_per_s"] for st in stats],
                         "tflops": [3 * fwd * st["samples_per_s"] / 1e12 for st in stats],
                         "final_loss": [st["loss"][-1] for st in stats], "loss_curve_member0": stats[0]["loss"]},
            "inference": {"samples_per_s": dtest.n * args.members / t_pred,
                          "tflops": fwd * dtest.n * args.members / t_pred / 1e12},
            "data_seconds": t_data, "train_data_solver_seconds": tr.seconds}
    print(json.dumps(line), flush=True)


def run_nn_step(args):
    """The surrogate network's training step alone (forward, backward, Adam) on resident random
    inputs: device-timed samples/s and tensor-core TFLOP/s against the measured bf16 peak."""
    import torch
    from se2dr_fork_gb300 import nn as N
    from se2dr_fork_gb300 import surrogate as SU
    torch.cuda.set_device(0)
    N.set_tensor_path(0 if args.mma_only else (2 if args.tc_all else 1))
    cfg = SU.net_config(args.nn_batch)
    net = N.Network(cfg, seed=0)
    stream = torch.cuda.Stream()
    net.set_stream(stream.cuda_stream)
    g = torch.Generator(device="cuda").manual_seed(0)
    with torch.cuda.stream(stream):
        x = torch.zeros(args.nn_batch, cfg.ny, cfg.nx, cfg.cin, device="cuda", dtype=torch.bfloat16)
        x[..., :6] = torch.randn(args.nn_batch, cfg.ny, cfg.nx, 6, device="cuda", generator=g).to(torch.bfloat16)
        t = torch.randn(args.nn_batch, cfg.nrec, cfg.nout, device="cuda", generator=g)
    for _ in range(args.warmup):
        net.loss_grad(x, t)
        net.adam_step(1e-4)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        net.loss_grad(x, t)
        net.adam_step(1e-4)
    ev1.record(stream)
    torch.cuda.synchronize()
    secs = ev0.elapsed_time(ev1) / 1e3
    fwd = SU.forward_flops(cfg)
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
        kind = "measured"
    except Exception:
        peak, kind = 1900.0, "fallback"
    sps = args.steps * args.nn_batch / secs
    tf = 3 * fwd * sps / 1e12
    paths = N.tensor_path_info()
    print(json.dumps({"metric": "surrogate training samples/s", "value": sps, "unit": "samples/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
                      "higher_is_better": True, "dtype": "bf16", "data": "synthetic",
                      "config": {"workload": "training step of the 4-layer, width-64, 16-mode operator on 128^2 "
                                             f"cells, batch {args.nn_batch}", "flops_per_sample": 3 * fwd,
                                 "row_gemms": ("mma.sync" if args.mma_only else "tcgen05" if args.tc_all
                                               else "tcgen05 except the 1x1 convolutions' shape")},
                      "gemm_launches": paths,
                      "roofline": {"bound": "tensor", "achieved": tf, "peak": peak, "unit": "TFLOP/s",
                                   "frac": tf / peak, "peak_kind": kind, "traffic": None}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp32_kahan", "fp32", "fp32_df", "fp64"], default="fp32_kahan")
    ap.add_argument("--mx", type=int, default=2048, help="elements per side (default: the 2048^2 workload)")
    ap.add_argument("--degree", type=int, default=4, help="polynomial degree of the single-solve run (default 4)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-df", action="store_true", help="skip the two-float FP32 leg")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-rows", type=int, default=32)
    ap.add_argument("--cpu-steps", type=int, default=6)
    ap.add_argument("--tile-config", type=int, default=-1, help="step-kernel tile configuration (-1: autotuned or default)")
    ap.add_argument("--autotune", action="store_true", help="measure every tile configuration first and cache the best")
    ap.add_argument("--sweep", action="store_true", help="degree sweep p = 1..8 at ~16M nodes instead of the headline run")
    ap.add_argument("--ensemble", action="store_true", help="batched ensemble of --shots shots instead of the headline run")
    ap.add_argument("--shots", type=int, default=256)
    ap.add_argument("--block", type=int, default=100, help="ensemble steps per CUDA graph")
    ap.add_argument("--ens-degree", type=int, default=0, help="give every ensemble shot this degree (0: as drawn)")
    ap.add_argument("--surrogate", action="store_true", help="surrogate training + serving instead of the headline run")
    ap.add_argument("--train", type=int, default=4000, help="surrogate training draws")
    ap.add_argument("--test", type=int, default=500, help="surrogate held-out requests (+10%% out of distribution)")
    ap.add_argument("--members", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--threshold", type=float, default=0.01)
    ap.add_argument("--serve-batch", type=int, default=250, help="requests per serving batch")
    ap.add_argument("--ladder-draws", type=int, default=1000, help="held-out draws the coarse-solver ladder re-solves")
    ap.add_argument("--nn-step", action="store_true", help="time the surrogate's training step alone")
    ap.add_argument("--nn-batch", type=int, default=32)
    ap.add_argument("--mma-only", action="store_true", help="surrogate GEMMs on the mma.sync kernel only")
    ap.add_argument("--tc-all", action="store_true", help="every qualifying surrogate row GEMM on tcgen05")
    ap.add_argument("--accuracy", action="store_true",
                    help="FP32 modes against FP64 over --steps steps (error table) instead of the headline run")
    ap.add_argument("--acc-tmax", type=float, default=0.0,
                    help="with --accuracy: run each mesh to this time instead of --steps steps")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.warmup < 3:
        args.warmup = 3
    if args.accuracy:
        run_accuracy(args)
    elif args.sweep:
        run_sweep(args)
    elif args.ensemble and args.impl == "ours":
        run_ensemble(args, rank, world)
    elif args.surrogate and args.impl == "ours":
        run_surrogate(args)
    elif args.nn_step and args.impl == "ours":
        run_nn_step(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
