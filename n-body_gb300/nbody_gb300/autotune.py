"""Autotuner for ensembles: the direct-sum / Barnes-Hut crossover size and
the direct-sum launch shape, measured on the GPU at hand and kept in a JSON
file.

For each size N of a grid it times ensembles of identical Plummer systems
(enough copies to fill the GPU) once all as direct sum and once all as
Barnes-Hut, in CUDA graphs, and takes the time per body-step; the crossover is
where Barnes-Hut becomes cheaper (interpolated in log N between grid points).
The launch shape is the fastest on a ragged direct-sum mix (N 256 .. 16,384),
picked first and used for the direct-sum timings. Both choices keep accuracy: the direct sum is exact up to FP32
rounding and every Barnes-Hut system keeps its theta.
"""
from __future__ import annotations

import json
import math
import os
import re
import time

import numpy as np

from .ensemble import PP_SHAPES, Ensemble

VERSION = 1
GRID = (256, 512, 1024, 2048, 4096, 8192, 16384, 32768)
PLUMMER = (50.0, 1.0, 20.0)


def default_path(device_name: str) -> str:
    safe = re.sub(r"[^A-Za-z0-9]+", "_", device_name).strip("_").lower() or "gpu"
    env = os.environ.get("NBODY_TUNE_FILE")
    return env or os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning", f"{safe}.json")


def _device_name(device: int) -> str:
    try:
        import torch

        return torch.cuda.get_device_name(device)
    except Exception:  # no torch / no device: the library still runs
        return "gpu"


def time_ensemble(sizes, mode, device=0, pp_shape="256x2", steps=3, graph_steps=3, seed=0) -> float:
    """Seconds per ensemble step (graph replay, after one warm-up replay)."""
    with Ensemble(crossover=0, device=device, pp_shape=pp_shape) as ens:
        for k, n in enumerate(sizes):
            sid = ens.add(int(n), 0.0035, 40.0, 0.25, mode=mode)
            ens.init_device(sid, "plummer", seed=seed + k, params=PLUMMER)
        ens.step(graph_steps, graph_steps)
        ens.sync()
        t0 = time.perf_counter()
        ens.step(steps, graph_steps)
        ens.sync()
        return (time.perf_counter() - t0) / steps


def crossover_from(grid, ns_pp: dict, ns_bh: dict) -> int:
    """The size from which Barnes-Hut is cheaper per body-step than the direct
    sum: the first grid point where it is, log-interpolated between that point
    and the one before; the grid's first point if Barnes-Hut always wins, twice
    its last if it never does."""
    grid = list(grid)
    if ns_bh[grid[0]] < ns_pp[grid[0]]:
        return int(grid[0])
    for a, b in zip(grid, grid[1:]):
        if ns_bh[b] < ns_pp[b]:
            # log(pp / bh) rises from <= 0 at a to > 0 at b
            ra, rb = math.log(ns_pp[a] / ns_bh[a]), math.log(ns_pp[b] / ns_bh[b])
            f = ra / (ra - rb)
            return int(round(math.exp(math.log(a) + f * (math.log(b) - math.log(a)))))
    return int(grid[-1] * 2)


def tune(device: int = 0, grid=GRID, bodies: int = 2_000_000, verbose: bool = False) -> dict:
    # launch shape first: a ragged direct-sum mix over the sizes the crossover can fall in
    rng = np.random.default_rng(1)
    mix = np.exp(rng.uniform(math.log(256), math.log(16384), 400)).astype(int)
    shapes = {s: time_ensemble(mix, "pp", device=device, pp_shape=s) for s in PP_SHAPES}
    best = min(shapes, key=shapes.get)
    if verbose:
        print("direct-sum shapes (ms per step):", {k: round(v * 1e3, 3) for k, v in shapes.items()}, flush=True)
    ns_pp, ns_bh = {}, {}
    for n in grid:
        copies = int(min(2048, max(8, bodies // n)))
        for mode, table in (("pp", ns_pp), ("bh", ns_bh)):
            t = time_ensemble([n] * copies, mode, device=device, pp_shape=best)
            table[n] = 1e9 * t / (copies * n)
        if verbose:
            print(f"N={n}: pp {ns_pp[n]:.3f} ns, bh {ns_bh[n]:.3f} ns per body-step", flush=True)
    # The crossover comes from the timings as stored (rounded), so that the file
    # reproduces it.
    ns_pp = {k: round(v, 4) for k, v in ns_pp.items()}
    ns_bh = {k: round(v, 4) for k, v in ns_bh.items()}
    crossover = crossover_from(grid, ns_pp, ns_bh)
    return {"version": VERSION, "device_name": _device_name(device), "crossover": int(crossover), "pp_shape": best,
            "ns_per_body_step": {"pp": {str(k): v for k, v in ns_pp.items()},
                                 "bh": {str(k): v for k, v in ns_bh.items()}},
            "pp_shape_ms_per_step": {k: round(v * 1e3, 4) for k, v in shapes.items()},
            "tuned_at": time.strftime("%Y-%m-%dT%H:%M:%S")}


def load_or_tune(device: int = 0, path: str | None = None, retune: bool = False, verbose: bool = False) -> dict:
    """The stored tuning for this GPU model, or a fresh one (then stored)."""
    name = _device_name(device)
    path = path or default_path(name)
    if not retune and os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        if d.get("version") == VERSION and d.get("device_name") == name:
            d["source"] = os.path.basename(path)
            return d
    d = tune(device=device, verbose=verbose)
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(d, f, indent=1)
        d["source"] = os.path.basename(path)
    except OSError:
        d["source"] = "not stored"
    return d


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="tune the ensemble crossover and direct-sum launch shape")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--retune", action="store_true")
    ap.add_argument("--path", default=None)
    a = ap.parse_args()
    print(json.dumps(load_or_tune(a.device, a.path, a.retune, verbose=True), indent=1))
