"""Autotuner for the step kernel's tile configuration.

The persistent FP32 kernel offers a few (elements per tile edge, threads per CTA)
configurations per polynomial degree (se2gpu_tile_configs).  Which is fastest
depends on the degree, the mesh size (tile count versus the SM count, halo
overhead) and the GPU, so it is measured: each configuration advances the real
problem for a few steps, timed with CUDA events on the solver's stream.  Results
are cached in a JSON file keyed by GPU name, degree, precision and mesh-size
class, and :func:`apply` looks them up for a new solver.
"""
from __future__ import annotations

import json
import math
import os
from typing import Dict, Optional

from .gpu import PRECISIONS, Solver

CACHE = os.environ.get("SE2GPU_TUNING", os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json"))


def _gpu_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def key(setup, precision: str) -> str:
    size_class = int(round(math.log2(max(1, setup.nnodes))))
    return f"{_gpu_name()}|p{setup.p}|{precision}|2^{size_class}"


def load() -> Dict[str, dict]:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def save(db: Dict[str, dict]):
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as f:
        json.dump(db, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def time_config(sol: Solver, config: int, steps: int, warmup: int = 2) -> float:
    """Mean device time per step (seconds) of one configuration."""
    import torch
    sol.set_tile_config(config)
    stream = torch.cuda.Stream()
    sol.set_stream(stream.cuda_stream)
    sol.advance(warmup)
    sol.traces()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    sol.advance(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    sol.traces()
    return e0.elapsed_time(e1) / 1e3 / steps


def tune(setup, precision: str = "fp32_kahan", steps: int = 10, write: bool = True) -> dict:
    """Measure every configuration on `setup`; return {config, edge, threads, seconds, all}."""
    sol = Solver(setup, precision, trace_capacity=2 * steps + 8)
    configs = sol.tile_configs()
    infos = [sol.tile_config_info(c) for c in range(len(configs))]
    times = [time_config(sol, c, steps) for c in range(len(configs))]
    sol.close()
    best = min(range(len(times)), key=lambda c: times[c])
    res = {"config": best, "edge": configs[best][0], "threads": configs[best][1], "seconds": times[best],
           "all": [dict(info, seconds=s) for info, s in zip(infos, times)]}
    if write:
        db = load()
        db[key(setup, precision)] = res
        save(db)
    return res


def lookup(setup, precision: str) -> Optional[int]:
    ent = load().get(key(setup, precision))
    return None if ent is None else int(ent["config"])


def apply(sol: Solver, precision: Optional[str] = None) -> int:
    """Select the cached best configuration for this solver (configuration 0 if none).
    `precision` defaults to the solver's own."""
    if precision is None:
        precision = {v: k for k, v in PRECISIONS.items()}[sol.precision]
    c = lookup(sol.setup, precision)
    if c is not None and c < len(sol.tile_configs()):
        sol.set_tile_config(c)
        return c
    return 0
