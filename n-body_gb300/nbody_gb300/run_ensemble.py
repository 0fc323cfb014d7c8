"""Command-line tool for users of the ensemble API: builds the ragged
Plummer ensemble on the device, steps it, and prints its step time and body
counts as one JSON line, so a user can check the batched solver on their own
GPU (and size an ensemble) without writing code:

    python -m nbody_gb300.run_ensemble [--systems 2048] [--steps 50] [--graph-steps 10]

Systems: Plummer clusters (a = 50, m = 1, truncated at 20 a), N log-uniform in
[256, 131072], eps^2 = 40, dt = 0.0035, theta = 0.5, direct sum below the
tuned crossover (or --crossover). It needs no host arrays: states are made by
the device generator. The same command, at a small --systems, is the one the
ensemble kernels are profiled with.
"""
from __future__ import annotations

import argparse
import json
import time

from . import Ensemble
from . import initializers as I


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m nbody_gb300.run_ensemble")
    ap.add_argument("--systems", type=int, default=2048)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--graph-steps", type=int, default=10)
    ap.add_argument("--crossover", type=int, default=None, help="default: the stored tuning")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--seed", type=int, default=2024)
    a = ap.parse_args(argv)
    if a.crossover is None:
        from .autotune import load_or_tune

        t = load_or_tune(a.device)
        crossover, shape = int(t["crossover"]), t["pp_shape"]
    else:
        crossover, shape = a.crossover, "128x2"
    sizes = I.ragged_sizes(a.systems, 256, 131072, seed=a.seed)
    with Ensemble(crossover=crossover, device=a.device, pp_shape=shape) as ens:
        for s, n in enumerate(sizes):
            sid = ens.add(int(n), 0.0035, 40.0, 0.25)
            ens.init_device(sid, "plummer", seed=7000 + s, params=(50.0, 1.0, 20.0))
        g = min(a.graph_steps, a.steps)
        ens.step(g, g)
        ens.sync()
        t0 = time.perf_counter()
        ens.step(a.steps, g)
        ens.sync()
        dt = time.perf_counter() - t0
        c = ens.counts()
    print(json.dumps({"systems": a.systems, "bodies": int(sizes.sum()), "steps": a.steps, "graph_steps": g,
                      "crossover": crossover, "pp_shape": shape, "seconds": round(dt, 4),
                      "ms_per_step": round(1e3 * dt / max(1, a.steps), 3),
                      "body_steps_per_s": float(sizes.sum()) * a.steps / dt, **c}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
