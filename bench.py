"""Benchmark of the per-step gravity solve on GB300; prints ONE JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload bh|discs|pp|ensemble|serving]
                    [--impl ours|reference]

Workloads (seeded synthetic inputs with the shapes the configurations name;
no public dataset is involved):
  bh (default): Barnes-Hut, N = 2^20 equal-mass Plummer sphere (a = 100,
       truncated at 20a, velocities from the Plummer distribution function),
       theta = 0.5, eps^2 = 40, dt = 0.0035 (the reference's -v 6 path).
       Metric: body-steps/s. The line also carries a "pp" object with the
       direct-sum workload measured the same way.
  discs: Barnes-Hut at scale, N = 2^24: two exponential discs of 8,388,607
       bodies (scale length 200, sech^2 height 20, circular velocities) plus a
       1e6 point mass each, 2,000 apart at relative speed 50, inclined 30 deg;
       theta = 0.6, eps^2 = 40, dt = 0.0035 (5 steps by default).
  pp : direct sum, N = 16,384 bodies uniform in a ball of radius 100, masses
       U[1, 10), v = 0, dt = 0.0035, eps^2 = 40 (the reference's -v 2 path).
       Metric: interactions/s (N^2 per step, 20 flop each by convention).

  ensemble: 2,048 independent Plummer clusters (a = 50, m = 1), N log-uniform
       in [256, 131072]; direct sum below the autotuned crossover, Barnes-Hut
       (theta = 0.5) above; eps^2 = 40, dt = 0.0035; steps replayed from CUDA
       graphs. Metric: sims/s (a sim = one system for 50 steps), beside the
       same systems stepped one at a time by the single-system solver. The
       default line nests it as "ensemble".
  serving: Poisson request streams (Plummer a = 100 or uniform ball R = 100,
       N log-uniform in [1024, 4194304], steps U[10, 500], dt in {0.001,
       0.0035}, eps^2 U[10, 40], theta = 0.5) served by the continuous-batching
       loop under a 150 GB budget, beside FIFO one-at-a-time single-system
       solves; p50 / p99 latency and sims/s. The default line nests one rate
       (100 req/s, 12 requests) as "serving", and the discs workload (5 steps,
       with its one-step CPU baseline) as "discs".

A "step" is one ParticleSolver::updateParticlePositions: forces + integrator.
value: K steps on HBM-resident state, timed with CUDA events on the launch
stream, L2 flushed (a 256 MiB write) between steps outside the event pair.
e2e:   the same steps through the C ABI's host-layout call (nbody_update_host)
with pinned host buffers, every step moving the reference layout in and out
(the library reads and writes page-locked buffers in place over the host link).
Multi-GPU: the path is replicated, not sharded ("replicas only"): under
torchrun every rank steps its own copy and value sums the ranks' work.

--impl reference times the reference's own CPU implementation of the path on
the host cores (the reference sources compiled headless when they are present
here, else this project's pinned C restatement of them), same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "n-body_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "PP interactions/s (%FP32 peak), BH body-steps/s; served sims/s + p99 vs plain"
PP_N, PP_DT, PP_EPS2 = 16384, 0.0035, 40.0
BH_N, BH_DT, BH_EPS2, BH_THETA2 = 1 << 20, 0.0035, 40.0, 0.25
DISCS_THETA2 = 0.36  # theta = 0.6
# Algorithmic bytes per body per step of the HBM-bound Barnes-Hut stages:
# bbox reads pos (16); keys read pos, write key + index (16 + 12); the sort reads
# keys once for the histograms (8) and moves key + index in and out in 8 passes
# (8 x 24); the gather reads index, pos, vel, acc, id and writes them (4 + 52 + 52);
# the build reads two neighbour keys per body and writes a 32-byte record (16 + 32);
# the upsweep reads a position and writes a partial sum per node (16 + 32).
BH_STAGE_BYTES = {"bh_bbox": 16, "bh_morton": 28, "bh_sort": 200, "bh_gather": 108, "bh_build": 48,
                  "bh_upsweep": 48}
FLOP_PER_INTERACTION = 20
L2_FLUSH_BYTES = 256 << 20
# Batched ragged ensemble: 2,048 Plummer clusters (a = 50, m = 1, truncated at
# 20 a), N log-uniform in [256, 131072]; a "sim" is one system run for 50 steps.
ENS_COUNT, ENS_LO, ENS_HI, ENS_STEPS, ENS_GRAPH = 2048, 256, 131072, 50, 10
ENS_PLUMMER = (50.0, 1.0, 20.0)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        d["source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0, "source": "fallback"}


def fp32_peak_tflops(sms: int, mhz: float) -> float:
    # 128 FP32 lanes per SM, an FMA counts 2 flop
    return sms * 128 * 2 * mhz * 1e6 / 1e12


class ClockSampler:
    """nvidia-smi samples (200 ms) taken while the GPU is under load."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.dev)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, util, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
            if len(parts) > 9:
                try:
                    util.append(float(parts[9]))
                except ValueError:
                    pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
               "samples": len(sm)}
        if util:
            out["util_pct"] = round(statistics.fmean(util), 1)
        return out


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init_dist(world, local):
    import torch

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return dist
    return None


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(dist, units: float, seconds: float) -> float:
    """Whole-job rate of independent replicas: the units all ranks processed
    divided by the slowest rank's time (its own time when run alone)."""
    if dist is None:
        return units / seconds
    import torch

    dev = "cuda" if torch.cuda.is_available() else "cpu"
    u = torch.tensor([units], dtype=torch.float64, device=dev)
    t = torch.tensor([seconds], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()) / float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def profile_value(kernel: str, key: str):
    """A number `key: value` from a committed ncu summary (profiles/<kernel>*.md), if any."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for fn in sorted(os.listdir(pdir)):
        if fn.startswith(kernel) and fn.endswith(".md"):
            with open(os.path.join(pdir, fn)) as f:
                m = re.search(key + r":\s*([0-9.eE+]+)", f.read())
            if m:
                return float(m.group(1))
    return None


def profile_traffic(kernel: str):
    """DRAM bytes per launch from a committed ncu summary (profiles/<kernel>*.md), if any."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for fn in sorted(os.listdir(pdir)):
        if fn.startswith(kernel) and fn.endswith(".md"):
            with open(os.path.join(pdir, fn)) as f:
                m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", f.read())
            if m:
                return float(m.group(1))
    return None


# ------------------------------------------------------------------ PP (ours)
def bench_pp(args, world, rank, local, dist):
    import torch

    import nbody_gb300 as nb
    from nbody_gb300 import initializers as I

    torch.cuda.set_device(local)
    n = PP_N
    pos, vel, mass = I.uniform_ball(n, seed=12345 + rank)
    system = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    solver = nb.ParticleSolverCUDA(PP_DT, PP_EPS2, n, mode="pp", device=local)
    # A dedicated (non-legacy) stream: the library launches on it and the
    # CUDA events below are recorded on it.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    solver.set_stream(stream.cuda_stream)
    solver.upload(system)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    cfg = solver.pp_config()
    launches_per_step = 1  # one pp_force_kernel launch per step (slices reduce inside it)

    def timed_steps(k, profile=False):
        evs = []
        for _ in range(k):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            solver.step(1)
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs)

    # warm-up (untimed), then a short soak so that the clock samples cover load
    timed_steps(max(3, args.warmup))
    sampler = ClockSampler(local)
    sampler.start()
    t_end = time.time() + 1.5
    while time.time() < t_end:
        timed_steps(20)
    barrier(dist)
    torch.cuda.synchronize()
    ms = timed_steps(args.steps)
    barrier(dist)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    value = replica_rate(dist, float(n) * n * args.steps, ms / 1e3)
    ms = max_over_ranks(dist, ms)
    sec = ms / 1e3
    interactions = float(n) * n * args.steps * world

    # dominant kernel alone: per-stage CUDA events on the launch stream
    solver.profile_enable(True)
    timed_steps(args.steps)
    prof = solver.profile_read()
    solver.profile_enable(False)
    f_ms, f_cnt = prof.get("pp_force", (0.0, 0))
    per_launch_s = f_ms / 1e3 / max(1, f_cnt)
    achieved_tflops = FLOP_PER_INTERACTION * float(n) * n / per_launch_s / 1e12
    pk = peaks()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    peak = fp32_peak_tflops(sms, float(pk.get("sm_max_mhz", 2070.0)))
    roofline = {"bound": "fp32", "achieved": round(achieved_tflops, 3), "peak": round(peak, 3), "unit": "TFLOP/s",
                "frac": round(achieved_tflops / peak, 4), "traffic": profile_traffic("pp_force"),
                "kernel": "pp_force_kernel", "kernel_ms_per_launch": round(per_launch_s * 1e3, 5),
                "peak_note": f"nominal FP32 FMA peak {sms} SMs x 128 lanes x 2 flop x {pk.get('sm_max_mhz')} MHz "
                             f"(max SM clock of {pk['source']} peaks file; no FP32 figure is measured there)",
                "stage_ms": {k: round(v[0] / max(1, v[1]), 5) for k, v in prof.items()}}
    if clocks.get("sm_mhz"):
        roofline["frac_at_median_clock"] = round(achieved_tflops / fp32_peak_tflops(sms, clocks["sm_mhz"]), 4)

    # end to end through the reference-facing call with pinned host buffers
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    hsys = nb.ParticleSystem(pin(pos.copy()), pin(vel.copy()), mass)
    hsys.masses = pin(hsys.masses)
    hsys.forces = pin(hsys.forces)
    hsys.accelerations = pin(hsys.accelerations)
    for _ in range(3):
        solver.update_particle_positions(hsys)
    torch.cuda.synchronize()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        solver.update_particle_positions(hsys)
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": interactions / e2e_s, "unit": "interactions/s", "h2d_bytes_per_step": 4 * 16 * n,
           "d2h_bytes_per_step": 4 * 16 * n, "ms_per_step": round(e2e_s * 1e3 / args.steps, 4),
           "api": "nbody_update_host (ParticleSolver::updateParticlePositions)"}

    line = {"metric": METRIC, "component": "PP interactions/s", "value": value, "unit": "interactions/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "direct-sum PP, N=16384 uniform ball R=100, m~U[1,10), v=0, dt=0.0035, "
                                   "eps2=40 (reference -v 2 path)", "n_bodies": n, "parallelism": "replicas",
                       "l2": "flushed between steps (256 MiB write, outside the event pair)",
                       "pp_launch": cfg},
            "clocks": clocks, "roofline": roofline, "e2e": e2e,
            "gpu_launches": launches_per_step * args.steps,
            "tflops_20flop": FLOP_PER_INTERACTION * interactions / sec / 1e12}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_pp()
    solver.close()
    torch.cuda.set_stream(torch.cuda.default_stream())
    return line


# ------------------------------------------------------------------ BH (ours)
def bench_bh(args, world, rank, local, dist):
    import torch

    import nbody_gb300 as nb
    from nbody_gb300 import initializers as I

    torch.cuda.set_device(local)
    discs = args.workload == "discs"
    if discs:
        pos, vel, mass = I.two_discs(seed=12345 + rank)
        theta2 = DISCS_THETA2
    else:
        pos, vel, mass = I.plummer(BH_N, a=100.0, seed=12345 + rank)
        theta2 = BH_THETA2
    n = len(mass)
    system = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    solver = nb.ParticleSolverCUDA(BH_DT, BH_EPS2, n, mode="bh", theta2=theta2, device=local)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    solver.set_stream(stream.cuda_stream)
    solver.upload(system)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def timed_steps(k):
        evs = []
        for _ in range(k):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            solver.step(1)
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs)

    timed_steps(max(3, args.warmup))
    solver.sync()
    sampler = ClockSampler(local)
    sampler.start()
    t_end = time.time() + 1.5
    while time.time() < t_end:
        timed_steps(5)
    barrier(dist)
    torch.cuda.synchronize()
    ms = timed_steps(args.steps)
    barrier(dist)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    solver.sync()
    value = replica_rate(dist, float(n) * args.steps, ms / 1e3)
    ms = max_over_ranks(dist, ms)
    sec = ms / 1e3

    # per-stage CUDA events on the launch stream (a separate pass)
    solver.profile_enable(True)
    timed_steps(args.steps)
    prof = solver.profile_read()
    solver.profile_enable(False)
    # work of the traversal (pairwise evaluations), counted in one more pass
    solver.bh_counters(True)
    timed_steps(1)
    pairs, visits = solver.bh_counters(False)
    pk = peaks()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32 = fp32_peak_tflops(sms, float(pk.get("sm_max_mhz", 2070.0)))
    t_ms, t_cnt = prof.get("bh_traverse", (0.0, 1))
    t_launch = t_ms / 1e3 / max(1, t_cnt)
    achieved = FLOP_PER_INTERACTION * pairs / t_launch / 1e12
    stages = {}
    for name, (sms_ms, cnt) in prof.items():
        per = sms_ms / max(1, cnt)
        st = {"ms": round(per, 4), "share": round(sms_ms / max(1e-9, sum(v[0] for v in prof.values())), 4)}
        if name in BH_STAGE_BYTES:
            gbs = BH_STAGE_BYTES[name] * n / (per / 1e3) / 1e9
            st.update({"bytes_per_body": BH_STAGE_BYTES[name], "achieved_gbs": round(gbs, 1),
                       "hbm_frac": round(gbs / pk["hbm_gbs"], 4)})
        stages[name] = st
    roofline = {"bound": "fp32", "achieved": round(achieved, 3), "peak": round(fp32, 3), "unit": "TFLOP/s",
                "frac": round(achieved / fp32, 4), "traffic": profile_traffic("bh_traverse"),
                "kernel": "traverse2_kernel" if os.environ.get("NBODY_BH_WALK") == "union" else "cell_walk_kernel",
                "kernel_ms_per_launch": round(t_launch * 1e3, 4),
                "work": {"pair_evaluations_per_step": pairs, "per_body": round(pairs / n, 1),
                         "warp_record_visits_per_step": visits,
                         "pair_evaluations_per_warp_visit": round(pairs / max(1, visits), 2)},
                "peak_note": f"nominal FP32 FMA peak ({sms} SMs x 128 lanes x 2 flop x {pk.get('sm_max_mhz')} MHz, "
                             f"{pk['source']} peaks file); 20 flop per pairwise evaluation, as for the direct sum. "
                             f"The traversal is latency/issue-bound; the other stages are graded against "
                             f"{pk['hbm_gbs']} GB/s HBM ({pk['source']}) in stages.",
                "stages": stages}

    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    hsys = nb.ParticleSystem(pin(pos.copy()), pin(vel.copy()), mass)
    hsys.masses = pin(hsys.masses)
    hsys.forces = pin(hsys.forces)
    hsys.accelerations = pin(hsys.accelerations)
    for _ in range(2):
        solver.update_particle_positions(hsys)
    torch.cuda.synchronize()
    barrier(dist)
    e2e_steps = max(1, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        solver.update_particle_positions(hsys)
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": float(n) * e2e_steps * world / e2e_s, "unit": "body-steps/s", "h2d_bytes_per_step": 4 * 16 * n,
           "d2h_bytes_per_step": 4 * 16 * n, "ms_per_step": round(e2e_s * 1e3 / e2e_steps, 3), "steps": e2e_steps,
           "api": "nbody_update_host (ParticleSolver::updateParticlePositions)"}
    # bbox, keys, sort (histogram, scan, 8 passes), gather, 7 build kernels and
    # the child table of the cell walk, the upsweep (one climbing launch below
    # 2^21 bodies; from there bucket centres, level count, level scatter and one
    # launch per octree level: 24), walk
    launches_per_step = 21 + (0 if os.environ.get("NBODY_BH_WALK") == "union" else 1) + \
        (1 if n < (1 << 21) else 24)
    line = {"metric": METRIC, "component": "BH body-steps/s", "value": value, "unit": "body-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": ("Barnes-Hut at scale, N=16777216: two exponential discs of 8388607 bodies "
                                    "(m=1, scale length 200, sech^2 height 20, circular velocities) + a 1e6 point "
                                    "mass each, 2000 apart, relative speed 50, inclined 30 deg; theta=0.6, eps2=40, "
                                    "dt=0.0035 (reference -v 6 path)") if discs else
                                   ("Barnes-Hut, N=1048576 equal-mass Plummer sphere a=100 (truncated at 20a, "
                                    "velocities from the Plummer DF), theta=0.5, eps2=40, dt=0.0035 "
                                    "(reference -v 6 path)"), "n_bodies": n, "parallelism": "replicas",
                       "l2": "flushed between steps (256 MiB write, outside the event pair)"},
            "clocks": clocks, "roofline": roofline, "e2e": e2e, "gpu_launches": launches_per_step * args.steps}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_discs(pos, vel, mass) if discs else cpu_baseline_bh()
    solver.close()
    torch.cuda.set_stream(torch.cuda.default_stream())
    return line


# ------------------------------------------------------------ ensemble (ours)
def bench_ensemble(args, world, rank, local, dist, steps=None):
    import torch

    import nbody_gb300 as nb
    from nbody_gb300 import autotune
    from nbody_gb300 import initializers as I

    torch.cuda.set_device(local)
    K = int(steps or args.steps)
    G = min(ENS_GRAPH, K)
    sizes = I.ragged_sizes(ENS_COUNT, ENS_LO, ENS_HI, seed=2024 + rank)
    total = int(sizes.sum())
    t_tune = time.perf_counter()
    tune = autotune.load_or_tune(local)
    t_tune = time.perf_counter() - t_tune
    X, shape = int(tune["crossover"]), tune["pp_shape"]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ens = nb.Ensemble(crossover=X, device=local, pp_shape=shape)
    ens.set_stream(stream.cuda_stream)
    ids = []
    for s_, n in enumerate(sizes):
        sid = ens.add(int(n), BH_DT, BH_EPS2, BH_THETA2)
        ens.init_device(sid, "plummer", seed=7000 + s_, params=ENS_PLUMMER)
        ids.append(sid)
    counts = ens.counts()
    pp_sizes = sizes[sizes < X]
    # initial states on the host (pinned), for the end-to-end pass
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    host0 = []
    for sid in ids:
        h = ens.download(sid)
        h.positions, h.velocities, h.accelerations, h.masses = (pin(h.positions), pin(h.velocities),
                                                                pin(h.accelerations), pin(h.masses))
        host0.append(h)

    ens.step(2 * G, G)  # warm-up; captures the graphs of both buffer parities
    ens.sync()
    sampler = ClockSampler(local)
    sampler.start()
    t_end = time.time() + 1.0
    while time.time() < t_end:
        ens.step(G, G)
        ens.sync()
    barrier(dist)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    ens.step(K, G)
    b.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    clocks = sampler.stop()
    ens.sync()
    value = replica_rate(dist, ENS_COUNT * K / ENS_STEPS, a.elapsed_time(b) / 1e3)
    ms = max_over_ranks(dist, a.elapsed_time(b))
    sec = ms / 1e3

    # per-stage times of one eager step (direct sum on the side stream, concurrent)
    ens.profile_enable(True)
    ens.step(2)
    prof = ens.profile_read()
    ens.profile_enable(False)
    pk = peaks()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32 = fp32_peak_tflops(sms, float(pk.get("sm_max_mhz", 2070.0)))
    pp_ms, pp_cnt = prof.get("pp_force", (0.0, 0))
    pp_launch = pp_ms / 1e3 / max(1, pp_cnt)
    pp_pairs = float(np.sum(pp_sizes.astype(np.float64) ** 2))
    pp_tf = FLOP_PER_INTERACTION * pp_pairs / pp_launch / 1e12 if pp_launch > 0 else 0.0
    bh_ms = sum(v[0] / max(1, v[1]) for k_, v in prof.items() if k_.startswith("bh_"))
    per_body = profile_value("pp_batch_kernel", "traffic_bytes_per_body")
    roofline = {"bound": "fp32", "achieved": round(pp_tf, 3), "peak": round(fp32, 3), "unit": "TFLOP/s",
                "frac": round(pp_tf / fp32, 4),
                "traffic": round(per_body * float(pp_sizes.sum())) if per_body else None,
                "traffic_note": "DRAM bytes per body of a smaller capture (profiles/pp_batch_kernel_ensemble_256_"
                                "systems.md) times this launch's direct-sum bodies",
                "kernel": "pp_batch_kernel",
                "kernel_ms_per_launch": round(pp_launch * 1e3, 4),
                "note": "the batched direct-sum kernel over the systems below the crossover (sum of N^2 pairs, "
                        "20 flop each); the Barnes-Hut stages of the other systems run beside it",
                "stages_ms_per_step": {k_: round(v[0] / max(1, v[1]), 4) for k_, v in prof.items()},
                "bh_stages_ms_per_step": round(bh_ms, 4)}

    # end to end through the public API: upload every system from pinned host
    # arrays, K steps, download every system
    out = [nb.ParticleSystem(*(pin(np.zeros((int(n), 4), np.float32)) for _ in range(2)),
                             pin(np.zeros((int(n), 4), np.float32)), pin(np.zeros((int(n), 4), np.float32)))
           for n in sizes]
    barrier(dist)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for sid, h in zip(ids, host0):
        ens.upload(sid, h)
    ens.step(K, G)
    for sid, o in zip(ids, out):
        ens.download(sid, o)
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": ENS_COUNT * world * K / ENS_STEPS / e2e_s, "unit": "sims/s",
           "h2d_bytes_per_step": int(4 * 16 * total / K), "d2h_bytes_per_step": int(4 * 16 * total / K),
           "seconds": round(e2e_s, 3),
           "api": "nbody_ensemble_upload x 2048, nbody_ensemble_step, nbody_ensemble_download x 2048"}
    launches = counts["launches_per_step"]
    ens.close()

    # the plain solver called one system at a time on the same GPU (same stream)
    k_plain = min(K, 10)
    solvers = []
    for s_, n in enumerate(sizes):
        mode = "pp" if n < X else "bh"
        sv = nb.ParticleSolverCUDA(BH_DT, BH_EPS2, int(n), mode=mode, theta2=BH_THETA2, device=local)
        sv.set_stream(stream.cuda_stream)
        sv.init_device("plummer", seed=7000 + s_, params=ENS_PLUMMER)
        solvers.append(sv)
    for sv in solvers:
        sv.step(1)
    torch.cuda.synchronize()
    a.record(stream)
    for sv in solvers:
        sv.step(k_plain)
    b.record(stream)
    torch.cuda.synchronize()
    for sv in solvers:
        sv.sync()
    plain_s = a.elapsed_time(b) / 1e3
    t_w = time.perf_counter()
    for sv in solvers:
        sv.step(k_plain)
    torch.cuda.synchronize()
    plain_wall = time.perf_counter() - t_w
    for sv in solvers:
        sv.close()
    plain = {"value": ENS_COUNT * k_plain / ENS_STEPS / plain_s, "unit": "sims/s",
             "wall_value": ENS_COUNT * k_plain / ENS_STEPS / plain_wall, "steps_per_system": k_plain,
             "how": "2048 single-system solvers (nbody_create, mode by the same crossover) on one stream, each "
                    "stepped k times before the next; CUDA events around the whole loop"}
    line = {"metric": METRIC, "component": "batched ensemble sims/s", "value": value, "unit": "sims/s",
            "n_gpus": world, "steps": K, "warmup": 2 * G, "ms_per_step": ms / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched ragged ensemble: 2048 Plummer clusters (a=50, m=1, truncated at 20a), "
                                   "N log-uniform in [256, 131072] (seed 2024); direct sum below the tuned "
                                   "crossover, Barnes-Hut theta=0.5 above; eps2=40, dt=0.0035; a sim = one system "
                                   "for 50 steps", "systems": ENS_COUNT, "bodies": total,
                       "crossover": X, "pp_shape": shape, "graph_steps": G,
                       "pp_systems": int(len(pp_sizes)), "bh_systems": int(ENS_COUNT - len(pp_sizes)),
                       "tuning": {k_: tune[k_] for k_ in ("source", "tuned_at") if k_ in tune},
                       "tuning_seconds": round(t_tune, 2), "parallelism": "replicas",
                       "l2": f"inputs larger than L2 ({total * 16 / 1e9:.2f} GB of positions)"},
            "body_steps_per_s": total * world * K / sec, "clocks": clocks, "roofline": roofline, "e2e": e2e,
            "plain_loop": plain, "speedup_vs_plain": round(value / plain["value"], 3),
            "gpu_launches": launches * K}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_ensemble(sizes, X)
    torch.cuda.set_stream(torch.cuda.default_stream())
    return line


# ------------------------------------------------------------- serving (ours)
SERVE_BUDGET = 150e9


BOUND_N = 1 << 20  # a single Barnes-Hut system of this size already fills the GPU (16,384 walk warps)


def _served_checks(reqs, served, alone):
    """Each served result against the same request run alone by the plain
    solver: Barnes-Hut bit for bit, direct sum within FP32 summation order."""
    bh_equal, n_bh, pp_err = 0, 0, 0.0
    for r in reqs:
        a, b = served.get(r.rid), alone.get(r.rid)
        if a is None or b is None or not (a.ok and b.ok):
            continue
        if a.mode == "bh":
            n_bh += 1
            bh_equal += int(np.array_equal(a.system.positions, b.system.positions) and
                            np.array_equal(a.system.velocities, b.system.velocities))
        else:
            ga, gb = a.system.accelerations[:, :3], b.system.accelerations[:, :3]
            rel = np.linalg.norm(ga - gb, axis=1) / np.maximum(np.linalg.norm(gb, axis=1), 1e-30)
            pp_err = max(pp_err, float(np.sqrt(np.mean(rel ** 2))))
    return {"bh_requests_bit_equal_alone": f"{bh_equal}/{n_bh}", "pp_requests_max_accel_rms_rel_vs_alone": pp_err}


def bench_serving(args, world, rank, local, dist, rates=(10.0, 100.0, 1000.0), count=None, pressure=True):
    """Config 5. The same requests (sizes, steps, seeds) arrive as Poisson
    streams at each rate. The plain solver serves them one at a time (FIFO),
    measured once in real time on the fastest stream with the phases of every
    service timed; its latencies at the slower rates follow from the FIFO
    recurrence over those service times (serving.fifo_replay). The lane server
    is measured in real time at every rate. GPU utilisation comes from
    nvidia-smi samples restricted to each arm."""
    import torch

    import nbody_gb300 as nb  # noqa: F401  (loads the library)
    from nbody_gb300 import autotune, serving

    torch.cuda.set_device(local)
    tune = autotune.load_or_tune(local)
    X, shape = int(tune["crossover"]), tune["pp_shape"]
    count = int(count or args.requests)
    fast = max(rates)
    base = serving.poisson_trace(count, rate=fast, seed=11 + rank)

    # warm-up (module load, first allocations), untimed
    serving.run_fifo_plain([serving.Request(rid=-1, n=4096, steps=3, dt=0.001, eps2=10.0)], device=local,
                           crossover=X, realtime=False)
    sampler = ClockSampler(local)
    sampler.start()
    fifo = serving.run_fifo_plain(base, device=local, crossover=X, realtime=True, timing=True)
    fifo_clocks = sampler.stop()
    service = {rid: r.completed - r.admitted for rid, r in fifo.items()}
    phases = {k: round(sum(r.timing.get(k, 0.0) for r in fifo.values() if r.timing), 3)
              for k in ("setup", "steps", "download", "teardown")}
    stages = {}
    for r in fifo.values():
        for k, v in ((r.timing or {}).get("stages") or {}).items():
            stages[k] = stages.get(k, 0.0) + v / 1e3
    t_fifo = sum(service.values())
    kernel_s = sum(stages.values())
    large = [r for r in base if r.n >= BOUND_N and fifo[r.rid].ok]
    t_large = sum(fifo[r.rid].timing["steps"] for r in large)
    bound = t_fifo / max(1e-9, t_large)
    fifo_info = {
        "service_s_total": round(t_fifo, 3), "phases_s": phases,
        "setup_teardown_s_per_request": round((phases["setup"] + phases["teardown"]) / max(1, len(fifo)), 5),
        "kernel_s": round(kernel_s, 3), "gpu_kernel_busy_frac": round(kernel_s / max(1e-9, t_fifo), 4),
        "walk_share_of_kernel_time": round(stages.get("bh_traverse", 0.0) / max(1e-9, kernel_s), 4),
        "stages_s": {k: round(v, 3) for k, v in sorted(stages.items())},
        "gpu_util_pct_nvidia_smi": fifo_clocks.get("util_pct"),
        "large_requests": len(large), "large_steps_s": round(t_large, 3),
        "large_work_share": round(sum(r.n * r.steps for r in large) / max(1, sum(r.n * r.steps for r in base)), 4),
        "clocks": fifo_clocks}
    per_rate = []
    for rate in rates:
        reqs = serving.poisson_trace(count, rate=rate, seed=11 + rank)
        with serving.LaneServer(budget_bytes=SERVE_BUDGET, device=local, crossover=X, pp_shape=shape,
                                max_chunk=10) as srv:
            srv.run_trace([serving.Request(rid=-1, n=4096, steps=3, dt=0.001, eps2=10.0)], realtime=False)
            sampler = ClockSampler(local)
            sampler.start()
            served = srv.run_trace(reqs, realtime=True)
            clocks = sampler.stop()
            stats = srv.stats
        plain = fifo if rate == fast else serving.fifo_replay(reqs, service)
        s_sum, p_sum = serving.summarize(served, reqs), serving.summarize(plain, reqs)
        entry = {"rate_req_per_s": rate, "served": s_sum, "plain_fifo": p_sum,
                 "plain_fifo_source": "measured" if rate == fast else "FIFO recurrence over the measured services",
                 "speedup_sims_per_s": round(s_sum["sims_per_s"] / max(1e-12, p_sum["sims_per_s"]), 3),
                 "p50_ratio_plain_over_served": round(p_sum["p50_latency_s"] / max(1e-12, s_sum["p50_latency_s"]), 3),
                 "p99_ratio_plain_over_served": round(p_sum["p99_latency_s"] / max(1e-12, s_sum["p99_latency_s"]), 3),
                 "max_in_flight": stats.max_in_flight, "chunks": stats.chunks,
                 "peak_footprint_gb": round(stats.peak_footprint / 1e9, 2),
                 "gpu_util_pct_nvidia_smi": clocks.get("util_pct"), "clocks": clocks}
        entry.update(_served_checks(reqs, served, fifo))
        per_rate.append(entry)
        del served
    out_pressure = None
    if pressure:
        # Admission under memory pressure: a budget of 1.5x the largest request's
        # footprint, so requests queue for memory as well as for the GPU.
        sub = base[: max(8, count // 2)]
        with serving.LaneServer(budget_bytes=1.0, device=local, crossover=X, pp_shape=shape, max_chunk=10) as srv:
            budget = int(1.5 * max(srv.footprint(r) for r in sub))
            srv.budget = budget
            t0 = time.perf_counter()
            served = srv.run_trace(sub, realtime=True)
            wall = time.perf_counter() - t0
            stats = srv.stats
        waits = [r.admitted - r.arrival for r in served.values() if r.ok]
        out_pressure = {"requests": len(sub), "rate_req_per_s": fast, "budget_gb": round(budget / 1e9, 2),
                        "completed": sum(r.ok for r in served.values()), "wall_s": round(wall, 3),
                        "max_in_flight": stats.max_in_flight, "peak_footprint_gb": round(stats.peak_footprint / 1e9, 2),
                        "admission_wait_p50_s": round(serving.percentile(waits, 50), 4),
                        "admission_wait_p99_s": round(serving.percentile(waits, 99), 4),
                        "summary": serving.summarize(served, sub)}
        out_pressure.update(_served_checks(sub, served, fifo))
        del served
    head = per_rate[-1] if per_rate[-1]["rate_req_per_s"] == fast else max(per_rate, key=lambda d: d["rate_req_per_s"])
    body_steps = sum(r.n * r.steps for r in base)
    return {"metric": METRIC, "component": "served sims/s", "value": head["served"]["sims_per_s"] * world,
            "unit": "sims/s", "n_gpus": world, "steps": None, "warmup": 1, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"serving: {count} requests per rate, Poisson arrivals; Plummer a=100 or uniform "
                                   f"ball R=100, N log-uniform in [1024, 4194304], steps U[10, 500], dt in "
                                   f"{{0.001, 0.0035}}, eps2 U[10, 40], theta=0.5; admission by HBM footprint under "
                                   f"150 GB; continuous batching in chunks of <= 10 steps, in 4 priority lanes by "
                                   f"N x steps; Barnes-Hut requests of >= {serving.SOLO_N} bodies one at a time on "
                                   f"the single-system solver in a fifth lane", "requests": count,
                       "rates": list(rates), "crossover": X,
                       "pp_shape": shape, "body_steps_per_trace": int(body_steps), "parallelism": "replicas"},
            "p50_latency_s": head["served"]["p50_latency_s"], "p99_latency_s": head["served"]["p99_latency_s"],
            "plain_fifo": head["plain_fifo"], "speedup_vs_plain": head["speedup_sims_per_s"],
            "attainable_speedup_bound": {
                "value": round(bound, 3),
                "how": f"FIFO service time of all requests / FIFO stepping time of the requests with N >= {BOUND_N} "
                       f"(each already fills the GPU: its walk has >= 16,384 warps). Batching cannot make those "
                       f"steps faster, so no schedule beats this ratio even if every smaller request were free."},
            "fifo_plain": fifo_info, "per_rate": per_rate, "memory_pressure": out_pressure,
            "clocks": head["clocks"],
            "e2e": {"value": head["served"]["sims_per_s"] * world, "unit": "sims/s",
                    "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(sum(4 * 16 * r.n for r in base)),
                    "note": "requests are generated on the device from their seeds; every result is downloaded "
                            "(4 vec4 arrays) before it counts as complete, inside the measured latency"}}


def cpu_baseline_ensemble(sizes, crossover, sample: int = 24, seed: int = 3):
    """The port on a random sample of the systems, one step each, scaled to the ensemble."""
    import pyoracle
    from nbody_gb300 import initializers as I

    pyoracle.build(reference=False)
    threads = cpu_threads()
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(sizes), size=min(sample, len(sizes)), replace=False)
    secs = 0.0
    for j in pick:
        n = int(sizes[j])
        pos, vel, mass = I.plummer(n, a=ENS_PLUMMER[0], seed=int(j))
        acc = np.zeros_like(pos)
        if n < crossover:
            secs += pyoracle.pp_run(pos, vel, acc, mass, BH_DT, BH_EPS2, 1, threads=threads)[4]
        else:
            secs += pyoracle.bh_run(pos, vel, acc, mass, BH_DT, BH_EPS2, 1, theta2=BH_THETA2, threads=threads,
                                    patched=True)[4]["seconds"]
    per_step_all = secs * len(sizes) / len(pick)
    return {"value": 1.0 / (per_step_all * ENS_STEPS), "unit": "sims/s", "cores": threads, "kind": "port",
            "sample": f"one step of each of {len(pick)} randomly chosen systems (-v 2 / -v 6 restated, {threads} "
                      f"threads), scaled to 2048 systems x 50 steps"}


def cpu_baseline_serving(count: int, sample: int = 6, seed: int = 11):
    """The port serving a random sample of the trace's requests (one step each, scaled by their step counts),
    scaled to the whole trace: requests per second of FIFO service on the host cores."""
    import pyoracle
    from nbody_gb300 import initializers as I
    from nbody_gb300 import serving

    pyoracle.build(reference=False)
    threads = cpu_threads()
    from nbody_gb300 import autotune

    with open(autotune.default_path("NVIDIA GB300")) as f:
        crossover = int(json.load(f)["crossover"])
    reqs = serving.poisson_trace(count, rate=100.0, seed=seed)
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(reqs), size=min(sample, len(reqs)), replace=False)
    secs = 0.0
    for j in pick:
        r = reqs[int(j)]
        if r.init == "plummer":
            pos, vel, mass = I.plummer(r.n, a=100.0, seed=int(j))
        else:
            pos, vel, mass = I.uniform_ball(r.n, radius=100.0, seed=int(j))
        acc = np.zeros_like(pos)
        if r.n < crossover:  # the same method as the served arm: direct sum below the crossover
            one = pyoracle.pp_run(pos, vel, acc, mass, r.dt, r.eps2, 1, threads=threads)[4]
        else:
            one = pyoracle.bh_run(pos, vel, acc, mass, r.dt, r.eps2, 1, theta2=r.theta2, threads=threads,
                                  patched=True)[4]["seconds"]
        secs += one * r.steps
    total = secs * len(reqs) / len(pick)
    return {"value": len(reqs) / total, "unit": "sims/s", "cores": threads, "kind": "port",
            "sample": f"one step (restated -v 2 below the crossover, -v 6 above, {threads} threads) of each of "
                      f"{len(pick)} randomly chosen requests, times its step count, scaled to the {len(reqs)}-request "
                      f"trace"}


def cpu_baseline_bh(budget_s: float = 15.0):
    import pyoracle
    from nbody_gb300 import initializers as I

    pyoracle.build(reference=False)
    threads = cpu_threads()
    pos, vel, mass = I.plummer(BH_N, a=100.0, seed=12345)
    acc = np.zeros_like(pos)
    r = pyoracle.bh_run(pos, vel, acc, mass, BH_DT, BH_EPS2, 1, theta2=BH_THETA2, threads=threads, patched=True)
    t1 = r[4]["seconds"]
    steps = max(1, min(10, int(budget_s / max(t1, 1e-3))))
    r = pyoracle.bh_run(pos, vel, acc, mass, BH_DT, BH_EPS2, steps, theta2=BH_THETA2, threads=threads, patched=True)
    return {"value": float(BH_N) * steps / r[4]["seconds"], "unit": "body-steps/s", "cores": threads,
            "kind": "port", "sample": f"{steps} full steps of the N=1048576 Plummer workload (-v 6 restated: "
                                      f"OpenMP tasks, integer node links, subtree regions sized from their "
                                      f"body counts; the reference's own -v 6 overflows its fixed regions on "
                                      f"this input), {threads} threads"}


def cpu_baseline_discs(pos, vel, mass):
    """One full -v 6 step (restated port) of the 16,777,216-body discs workload on the host cores."""
    import pyoracle

    pyoracle.build(reference=False)
    threads = cpu_threads()
    acc = np.zeros_like(pos)
    r = pyoracle.bh_run(pos, vel, acc, mass, BH_DT, BH_EPS2, 1, theta2=DISCS_THETA2, threads=threads, patched=True)
    return {"value": float(len(mass)) / r[4]["seconds"], "unit": "body-steps/s", "cores": threads, "kind": "port",
            "sample": f"1 full step of the N=16777216 discs workload (-v 6 restated: OpenMP tasks, integer node "
                      f"links, subtree regions sized from their body counts), theta=0.6, {threads} threads"}


def cpu_kind():
    import pyoracle

    return "reference" if pyoracle.ref_available() else "port"


def cpu_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def cpu_pp_step_seconds(pos, vel, mass, steps, threads):
    import pyoracle

    acc = np.zeros_like(pos)
    if pyoracle.ref_available():
        return pyoracle.ref_run(2, pos, vel, acc, mass, PP_DT, PP_EPS2, steps, threads=threads)[4]["seconds"]
    return pyoracle.pp_run(pos, vel, acc, mass, PP_DT, PP_EPS2, steps, threads=threads)[4]


def cpu_baseline_pp(budget_s: float = 12.0):
    import pyoracle
    from nbody_gb300 import initializers as I

    pyoracle.build(reference=False)
    threads = cpu_threads()
    pos, vel, mass = I.uniform_ball(PP_N, seed=12345)
    t1 = cpu_pp_step_seconds(pos, vel, mass, 1, threads)
    steps = max(1, min(100, int(budget_s / max(t1, 1e-3))))
    secs = cpu_pp_step_seconds(pos, vel, mass, steps, threads)
    return {"value": float(PP_N) * PP_N * steps / secs, "unit": "interactions/s", "cores": threads,
            "kind": cpu_kind(), "sample": f"{steps} full steps of the N=16384 workload (-v 2 OpenMP, "
                                          f"{threads} threads)"}


def bench_reference(args, world, rank):
    if rank != 0:
        return None
    import pyoracle
    from nbody_gb300 import initializers as I

    pyoracle.build(reference=False)
    threads = cpu_threads()
    if args.workload == "pp":
        pos, vel, mass = I.uniform_ball(PP_N, seed=12345)
        for _ in range(args.warmup):
            cpu_pp_step_seconds(pos, vel, mass, 1, threads)
        # each step is one full -v 2 step; the count is bounded to keep the run within minutes
        t1 = cpu_pp_step_seconds(pos, vel, mass, 1, threads)
        steps = max(1, min(args.steps, int(120.0 / max(t1, 1e-3))))
        secs = cpu_pp_step_seconds(pos, vel, mass, steps, threads)
        value = float(PP_N) * PP_N * steps / secs
        kind = cpu_kind()
        unit, comp = "interactions/s", "PP interactions/s"
        workload = ("direct-sum PP, N=16384 uniform ball R=100, m~U[1,10), v=0, dt=0.0035, eps2=40 "
                    "(reference -v 2 path)")
        sample = f"{steps} full steps (-v 2 OpenMP, {threads} threads)"
        n = PP_N
    elif args.workload in ("ensemble", "serving"):
        if args.workload == "ensemble":
            from nbody_gb300 import autotune

            tune_path = autotune.default_path("NVIDIA GB300")
            with open(tune_path) as f:
                X = int(json.load(f)["crossover"])
            sizes = I.ragged_sizes(ENS_COUNT, ENS_LO, ENS_HI, seed=2024)
            cb = cpu_baseline_ensemble(sizes, X)
            workload = ("batched ragged ensemble: 2048 Plummer clusters (a=50, m=1), N log-uniform in [256, 131072]; "
                        "direct sum below the crossover, Barnes-Hut theta=0.5 above; a sim = one system for 50 steps")
            n = int(sizes.sum())
        else:
            cb = cpu_baseline_serving(args.requests)
            workload = ("serving trace: Plummer a=100 or uniform ball R=100, N log-uniform in [1024, 4194304], steps "
                        "U[10, 500]; requests served one at a time on the host cores")
            n = None
        value, unit, kind, sample = cb["value"], cb["unit"], cb["kind"], cb["sample"]
        comp, steps, secs = ("batched ensemble sims/s" if args.workload == "ensemble" else "served sims/s"), 1, 1.0
    elif args.workload == "discs":
        pos, vel, mass = I.two_discs(seed=12345)
        acc = np.zeros_like(pos)
        # one warm-up step, then at most two timed full -v 6 steps (each ~30 s)
        pyoracle.bh_run(pos, vel, acc, mass, BH_DT, BH_EPS2, 1, theta2=DISCS_THETA2, threads=threads, patched=True)
        steps = max(1, min(args.steps, 2))
        r = pyoracle.bh_run(pos, vel, acc, mass, BH_DT, BH_EPS2, steps, theta2=DISCS_THETA2, threads=threads,
                            patched=True)
        secs = r[4]["seconds"]
        n = len(mass)
        value = float(n) * steps / secs
        kind = "port"
        unit, comp = "body-steps/s", "BH body-steps/s"
        workload = ("Barnes-Hut at scale, N=16777216: two exponential discs of 8388607 bodies (m=1, scale length "
                    "200, sech^2 height 20, circular velocities) + a 1e6 point mass each, 2000 apart, relative speed "
                    "50, inclined 30 deg; theta=0.6, eps2=40, dt=0.0035 (reference -v 6 path)")
        sample = (f"{steps} full steps after 1 warm-up step (-v 6 restated with integer node links and subtree "
                  f"regions sized from their body counts), {threads} threads")
    else:
        pos, vel, mass = I.plummer(BH_N, a=100.0, seed=12345)
        acc = np.zeros_like(pos)
        # warm-up, then a bounded number of full -v 6 steps (each a few seconds)
        r = pyoracle.bh_run(pos, vel, acc, mass, BH_DT, BH_EPS2, 1, theta2=BH_THETA2, threads=threads,
                            patched=True)
        t1 = r[4]["seconds"]
        steps = max(1, min(args.steps, int(120.0 / max(t1, 1e-3))))
        r = pyoracle.bh_run(pos, vel, acc, mass, BH_DT, BH_EPS2, steps, theta2=BH_THETA2, threads=threads,
                            patched=True)
        secs = r[4]["seconds"]
        value = float(BH_N) * steps / secs
        kind = "port"
        unit, comp = "body-steps/s", "BH body-steps/s"
        workload = ("Barnes-Hut, N=1048576 equal-mass Plummer sphere a=100 (truncated at 20a, velocities from "
                    "the Plummer DF), theta=0.5, eps2=40, dt=0.0035 (reference -v 6 path)")
        sample = (f"{steps} full steps (-v 6 restated with integer node links and subtree regions sized from "
                  f"their body counts; the reference's own -v 6 overflows its fixed regions on this input), "
                  f"{threads} threads")
        n = BH_N
    per_step = None if args.workload in ("ensemble", "serving") else secs * 1e3 / steps
    return {"impl": "reference", "metric": METRIC, "component": comp, "value": value, "unit": unit,
            "n_gpus": world, "steps": steps, "warmup": args.warmup, "ms_per_step": per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload, "n_bodies": n, "parallelism": "host cores"},
            "cpu_baseline": {"value": value, "unit": unit, "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", choices=["bh", "discs", "pp", "ensemble", "serving"], default="bh")
    ap.add_argument("--requests", type=int, default=48, help="requests per rate of the serving workload")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-pp", action="store_true", help="leave the nested direct-sum measurement out")
    ap.add_argument("--no-ensemble", action="store_true", help="leave the nested ensemble measurement out")
    ap.add_argument("--no-serving", action="store_true", help="leave the nested serving measurement out")
    ap.add_argument("--no-discs", action="store_true", help="leave the nested 16M discs measurement out")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_env()
    if args.impl == "reference":
        line = bench_reference(args, world, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    import nbody_gb300
    from nbody_gb300 import build as nbuild

    if not os.path.exists(nbody_gb300.LIB_PATH):
        nbuild.build()
    dist = init_dist(world, local)
    if args.workload == "pp":
        line = bench_pp(args, world, rank, local, dist)
    elif args.workload == "ensemble":
        line = bench_ensemble(args, world, rank, local, dist)
    elif args.workload == "serving":
        line = bench_serving(args, world, rank, local, dist)
    else:
        line = bench_bh(args, world, rank, local, dist)
        if not args.no_pp and args.workload == "bh":
            pp_args = argparse.Namespace(**vars(args))
            pp_args.steps = 100
            pp = bench_pp(pp_args, world, rank, local, dist)
            line["pp"] = {k: pp[k] for k in ("component", "value", "unit", "steps", "ms_per_step", "roofline",
                                             "e2e", "clocks", "gpu_launches", "config", "cpu_baseline")
                          if k in pp}
        if not args.no_ensemble and args.workload == "bh":
            en = bench_ensemble(args, world, rank, local, dist, steps=ENS_STEPS)
            line["ensemble"] = {k: en[k] for k in ("component", "value", "unit", "steps", "ms_per_step", "roofline",
                                                   "e2e", "clocks", "gpu_launches", "config", "plain_loop",
                                                   "speedup_vs_plain", "body_steps_per_s", "cpu_baseline")
                                if k in en}
        if not args.no_discs and args.workload == "bh":
            d_args = argparse.Namespace(**vars(args))
            d_args.workload = "discs"
            d_args.steps = min(args.steps, 5)
            dl = bench_bh(d_args, world, rank, local, dist)
            line["discs"] = {k: dl[k] for k in ("component", "value", "unit", "steps", "ms_per_step", "roofline",
                                                "e2e", "clocks", "gpu_launches", "config", "cpu_baseline")
                             if k in dl}
        if not args.no_serving and args.workload == "bh":
            sv = bench_serving(args, world, rank, local, dist)
            line["serving"] = {k: sv[k] for k in ("component", "value", "unit", "p50_latency_s", "p99_latency_s",
                                                  "plain_fifo", "speedup_vs_plain", "attainable_speedup_bound",
                                                  "fifo_plain", "per_rate", "memory_pressure", "config", "e2e")
                               if k in sv}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
