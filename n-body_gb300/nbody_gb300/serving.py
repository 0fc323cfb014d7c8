"""Serving: a request loop with continuous batching over an ensemble.

A request carries an initial state (explicit host arrays, or a seeded
generator run on the device), N, dt, eps^2, theta and a step count. The server
keeps every admitted request's state resident in HBM inside one Ensemble,
admits waiting requests in arrival order while their device footprint fits the
memory budget, steps all admitted requests together in chunks of at most
`max_chunk` steps (a chunk never runs past the soonest finish), and between
chunks retires finished requests (download, remove) and folds new arrivals
into the next launch. A request's result does not depend on what else was in
flight: ensembles compute every system on its own.

`run_fifo_plain` is the comparison point: the single-system solver
(nbody_create) serving the same requests one at a time in arrival order.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import NBodyError, ParticleSolverCUDA, ParticleSystem
from .ensemble import Ensemble


@dataclass
class Request:
    rid: int
    n: int
    steps: int
    dt: float
    eps2: float
    theta2: float = 0.25
    init: str = "plummer"            # a device initialiser kind, or "state"
    params: tuple | None = None      # initialiser parameters
    seed: int = 0
    state: ParticleSystem | None = None  # explicit initial state (init == "state")
    arrival: float = 0.0             # seconds after the start of the trace


@dataclass
class Result:
    rid: int
    ok: bool
    mode: str = ""
    system: ParticleSystem | None = None
    error: str = ""
    arrival: float = 0.0
    admitted: float = 0.0
    completed: float = 0.0
    timing: dict | None = None  # run_fifo_plain(timing=True): phases of the service, seconds

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


@dataclass
class _Active:
    req: Request
    sid: int
    left: int
    footprint: int
    admitted: float
    mode: str = ""


@dataclass
class ServerStats:
    chunks: int = 0
    steps: int = 0
    relayouts: int = 0
    max_in_flight: int = 0
    peak_footprint: int = 0
    busy_seconds: float = 0.0
    in_flight_samples: list = field(default_factory=list)


def percentile(xs, q) -> float:
    return float(np.percentile(np.asarray(xs, np.float64), q)) if len(xs) else float("nan")


class Server:
    """Continuous batching in one shared ensemble: every admitted request steps
    in every chunk (processor sharing)."""

    def __init__(self, budget_bytes: float = 150e9, device: int = 0, crossover: int | None = None,
                 pp_shape: str | None = None, max_chunk: int = 10, keep_results: bool = True, ensemble=None):
        """`ensemble` replaces the device ensemble (any object with the
        Ensemble methods; used to test the loop without a GPU)."""
        if ensemble is not None and crossover is None:
            crossover = ensemble.crossover
        if ensemble is None and (crossover is None or pp_shape is None):
            from .autotune import load_or_tune

            t = load_or_tune(device)
            crossover = t["crossover"] if crossover is None else crossover
            pp_shape = t["pp_shape"] if pp_shape is None else pp_shape
        self.budget = int(budget_bytes)
        self.crossover = int(crossover)
        self.max_chunk = int(max_chunk)
        self.keep_results = keep_results
        self.ens = ensemble if ensemble is not None else Ensemble(crossover=self.crossover, device=device,
                                                                  pp_shape=pp_shape)
        self.stats = ServerStats()

    def close(self) -> None:
        self.ens.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def footprint(self, req: Request) -> int:
        mode = "pp" if req.n < self.crossover else "bh"
        # a re-layout holds the old and the new packed state for a moment
        return 2 * self.ens.footprint(req.n, mode)

    def _admit(self, req: Request, now: float) -> _Active:
        ens = self.ens
        sid = ens.add(req.n, req.dt, req.eps2, req.theta2)
        try:
            if req.init == "state":
                if req.state is None or req.state.n != req.n:
                    raise ValueError("request state missing or of the wrong size")
                ens.upload(sid, req.state)
            else:
                ens.init_device(sid, req.init, seed=req.seed, params=req.params)
        except Exception:
            ens.remove(sid)
            raise
        return _Active(req, sid, req.steps, self.footprint(req), now, ens.info(sid)[0])

    def run_trace(self, requests, realtime: bool = True, clock=time.perf_counter):
        """Serves `requests` (arrival times relative to the start). With
        realtime, a request becomes visible when the wall clock passes its
        arrival; otherwise all are visible at once. Returns results by rid."""
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        queue: list[Request] = []
        active: list[_Active] = []
        results: dict[int, Result] = {}
        used = 0
        t0 = clock()
        now = lambda: clock() - t0  # noqa: E731
        st = self.stats
        while pending or queue or active:
            t = now()
            while pending and (not realtime or pending[0].arrival <= t):
                queue.append(pending.pop(0))
            # admission in arrival order while the footprint fits
            changed = False
            while queue:
                req = queue[0]
                fp = self.footprint(req)
                if fp > self.budget:
                    queue.pop(0)
                    results[req.rid] = Result(req.rid, False, error="larger than the memory budget",
                                              arrival=req.arrival, admitted=t, completed=now())
                    continue
                if used + fp > self.budget:
                    break
                queue.pop(0)
                try:
                    act = self._admit(req, now())
                except (NBodyError, ValueError) as e:
                    results[req.rid] = Result(req.rid, False, error=str(e), arrival=req.arrival, admitted=now(),
                                              completed=now())
                    continue
                active.append(act)
                used += act.footprint
                changed = True
            if changed:
                st.relayouts += 1
            st.max_in_flight = max(st.max_in_flight, len(active))
            st.peak_footprint = max(st.peak_footprint, used)
            if not active:
                if pending and realtime:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - now())))
                continue
            k = min(self.max_chunk, min(a.left for a in active))
            tb = clock()
            try:
                self.ens.step(k)
                self.ens.sync()
            except NBodyError as e:
                # a failed step: every request in flight fails, the server goes on
                for a in active:
                    results[a.req.rid] = Result(a.req.rid, False, a.mode, error=str(e), arrival=a.req.arrival,
                                                admitted=a.admitted, completed=now())
                    self.ens.remove(a.sid)
                active, used = [], 0
                continue
            st.busy_seconds += clock() - tb
            st.chunks += 1
            st.steps += k
            st.in_flight_samples.append(len(active))
            still = []
            for a in active:
                a.left -= k
                if a.left > 0:
                    still.append(a)
                    continue
                system = self.ens.download(a.sid) if self.keep_results else None
                self.ens.remove(a.sid)
                used -= a.footprint
                results[a.req.rid] = Result(a.req.rid, True, a.mode, system, arrival=a.req.arrival,
                                            admitted=a.admitted, completed=now())
            active = still
        return results


# Lane bounds in body-steps (N x steps) of a request's whole run.
LANE_BOUNDS = (2e7, 2e8, 2e9)
# Barnes-Hut requests from this size on run alone, one at a time, in a lane of
# their own: one such system already fills the GPU (its walk has >= 16,384
# warps), so batching it gains nothing, and the single-system solver's walk is
# faster than the ensemble's on it (GB300, a 2^20 Plummer sphere: 4.6 against
# 5.0 ms a step). Their results are the single-system solver's bit for bit.
SOLO_N = 1 << 20


class _Solo:
    """The lane of the largest Barnes-Hut requests: one request at a time on
    the single-system solver, stepped in chunks on the lane's stream."""

    def __init__(self, stream):
        self.stream = stream
        self.incoming: list[tuple] = []  # (request, footprint, admitted at)
        self.solver = None
        self.active: _Active | None = None
        self.event = None
        self.chunk = 0


class _Lane:
    def __init__(self, index, ens, stream):
        self.index = index
        self.ens = ens
        self.stream = stream
        self.active: list[_Active] = []
        self.incoming: list[tuple] = []  # admitted (memory reserved), joins at the lane's next chunk
        self.event = None  # set while a chunk is in flight
        self.chunk = 0


class LaneServer:
    """Continuous batching in priority lanes. A request joins the lane of its
    total work (N x steps; bounds LANE_BOUNDS), each lane is an ensemble on
    its own CUDA stream, smaller work on higher stream priority. Every lane
    with work has a chunk in flight, so lanes overlap on the GPU while the block
    scheduler favours the small ones; finished chunks are noticed by polling
    their events, their finished requests retired and arrivals admitted
    (arrival order, shared memory budget). Barnes-Hut requests of solo_n
    bodies or more run one at a time on the single-system solver in a lane of
    their own, at the lowest priority, beside the batched lanes. Results do
    not depend on lanes: every system is computed on its own."""

    def __init__(self, budget_bytes: float = 150e9, device: int = 0, crossover: int | None = None,
                 pp_shape: str | None = None, max_chunk: int = 10, keep_results: bool = True,
                 bounds=LANE_BOUNDS, solo_n: int | None = SOLO_N):
        import torch

        if crossover is None or pp_shape is None:
            from .autotune import load_or_tune

            t = load_or_tune(device)
            crossover = t["crossover"] if crossover is None else crossover
            pp_shape = t["pp_shape"] if pp_shape is None else pp_shape
        self.budget = int(budget_bytes)
        self.crossover = int(crossover)
        self.pp_shape = pp_shape
        self.device = device
        self.max_chunk = int(max_chunk)
        self.keep_results = keep_results
        self.bounds = tuple(bounds)
        self.stats = ServerStats()
        lo, hi = torch.cuda.Stream.priority_range()  # e.g. (0, -5): lower is more urgent
        nl = len(self.bounds) + 1
        self.lanes = []
        for k in range(nl):
            prio = hi + round((lo - hi) * k / max(1, nl - 1)) if lo != hi else lo
            stream = torch.cuda.Stream(device=device, priority=int(prio))
            ens = Ensemble(crossover=self.crossover, device=device, pp_shape=pp_shape)
            ens.set_stream(stream.cuda_stream)
            self.lanes.append(_Lane(k, ens, stream))
        self.solo_n = None if solo_n is None else int(solo_n)
        self.solo = _Solo(torch.cuda.Stream(device=device, priority=int(lo))) if self.solo_n else None

    def close(self) -> None:
        for lane in self.lanes:
            lane.ens.close()
        if self.solo is not None and self.solo.solver is not None:
            self.solo.solver.close()
            self.solo.solver = None

    def is_solo(self, req: Request) -> bool:
        return self.solo is not None and req.n >= max(self.solo_n, self.crossover)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def footprint(self, req: Request) -> int:
        mode = "pp" if req.n < self.crossover else "bh"
        return 2 * Ensemble.footprint(req.n, mode)

    def lane_of(self, req: Request) -> int:
        work = float(req.n) * req.steps
        for k, b in enumerate(self.bounds):
            if work < b:
                return k
        return len(self.bounds)

    def run_trace(self, requests, realtime: bool = True, clock=time.perf_counter):
        import torch

        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        queue: list[Request] = []
        results: dict[int, Result] = {}
        used = 0
        t0 = clock()
        now = lambda: clock() - t0  # noqa: E731
        st = self.stats

        def fail(a, lane, err):
            results[a.req.rid] = Result(a.req.rid, False, a.mode, error=err, arrival=a.req.arrival,
                                        admitted=a.admitted, completed=now())
            lane.ens.remove(a.sid)

        solo = self.solo

        def solo_end(err=None):
            a = solo.active
            system = None
            if err is None and self.keep_results:
                z = np.zeros((a.req.n, 4), np.float32)
                system = ParticleSystem(z, z.copy(), np.zeros(a.req.n, np.float32), z.copy())
                try:
                    solo.solver.download(system, masses=True)
                except NBodyError as e:
                    err = str(e)
            if solo.solver is not None:
                solo.solver.close()
            results[a.req.rid] = Result(a.req.rid, err is None, "bh", system if err is None else None,
                                        error=err or "", arrival=a.req.arrival, admitted=a.admitted,
                                        completed=now())
            solo.solver, solo.active, solo.event = None, None, None
            return a.footprint

        def solo_busy():
            return solo is not None and (solo.active is not None or solo.incoming)

        while pending or queue or any(l.active or l.incoming for l in self.lanes) or solo_busy():
            t = now()
            while pending and (not realtime or pending[0].arrival <= t):
                queue.append(pending.pop(0))
            # the solo lane: a finished chunk moves its request on or retires it
            if solo is not None and solo.event is not None and solo.event.query():
                solo.event = None
                solo.active.left -= solo.chunk
                if solo.active.left <= 0:
                    used -= solo_end()
            # retire lanes whose chunk has finished
            for lane in self.lanes:
                if lane.event is None or not lane.event.query():
                    continue
                lane.event = None
                k = lane.chunk
                try:
                    lane.ens.sync()
                except NBodyError as e:
                    for a in lane.active:
                        fail(a, lane, str(e))
                        used -= a.footprint
                    lane.active = []
                    continue
                still = []
                for a in lane.active:
                    a.left -= k
                    if a.left > 0:
                        still.append(a)
                        continue
                    system = lane.ens.download(a.sid) if self.keep_results else None
                    lane.ens.remove(a.sid)
                    used -= a.footprint
                    results[a.req.rid] = Result(a.req.rid, True, a.mode, system, arrival=a.req.arrival,
                                                admitted=a.admitted, completed=now())
                lane.active = still
            # admission in arrival order under the shared memory budget; the
            # request joins its lane's ensemble when the lane is idle
            while queue:
                req = queue[0]
                fp = self.footprint(req)
                if fp > self.budget:
                    queue.pop(0)
                    results[req.rid] = Result(req.rid, False, error="larger than the memory budget",
                                              arrival=req.arrival, admitted=now(), completed=now())
                    continue
                if used + fp > self.budget:
                    break
                queue.pop(0)
                if self.is_solo(req):
                    solo.incoming.append((req, fp, now()))
                else:
                    self.lanes[self.lane_of(req)].incoming.append((req, fp, now()))
                used += fp
            # the solo lane, when idle, starts its next request; one chunk at a time
            if solo is not None and solo.event is None:
                if solo.active is None and solo.incoming:
                    req, fp, t_adm = solo.incoming.pop(0)
                    solo.active = _Active(req, -1, req.steps, fp, t_adm, "bh")
                    try:
                        if req.init == "state" and (req.state is None or req.state.n != req.n):
                            raise ValueError("request state missing or of the wrong size")
                        solo.solver = ParticleSolverCUDA(req.dt, req.eps2, req.n, mode="bh", theta2=req.theta2,
                                                         device=self.device)
                        solo.solver.set_stream(solo.stream.cuda_stream)
                        if req.init == "state":
                            solo.solver.upload(req.state)
                        else:
                            solo.solver.init_device(req.init, seed=req.seed, params=req.params)
                    except (NBodyError, ValueError) as e:
                        used -= solo_end(str(e))
                if solo.active is not None:
                    k = min(self.max_chunk, solo.active.left)
                    try:
                        solo.solver.step(k)
                        ev = torch.cuda.Event()
                        ev.record(solo.stream)
                        solo.event, solo.chunk = ev, k
                        st.chunks += 1
                        st.steps += k
                    except NBodyError as e:
                        used -= solo_end(str(e))
            # an idle lane takes its incoming requests, then every idle lane with
            # work launches a chunk
            launched = False
            for lane in self.lanes:
                if lane.event is not None:
                    continue
                ens = lane.ens
                for req, fp, t_adm in lane.incoming:
                    try:
                        sid = ens.add(req.n, req.dt, req.eps2, req.theta2)
                        try:
                            if req.init == "state":
                                if req.state is None or req.state.n != req.n:
                                    raise ValueError("request state missing or of the wrong size")
                                ens.upload(sid, req.state)
                            else:
                                ens.init_device(sid, req.init, seed=req.seed, params=req.params)
                        except Exception:
                            ens.remove(sid)
                            raise
                    except (NBodyError, ValueError) as e:
                        results[req.rid] = Result(req.rid, False, error=str(e), arrival=req.arrival,
                                                  admitted=t_adm, completed=now())
                        used -= fp
                        continue
                    lane.active.append(_Active(req, sid, req.steps, fp, t_adm, ens.info(sid)[0]))
                lane.incoming = []
                if not lane.active:
                    continue
                k = min(self.max_chunk, min(a.left for a in lane.active))
                try:
                    lane.ens.step(k)
                except NBodyError as e:
                    for a in lane.active:
                        fail(a, lane, str(e))
                        used -= a.footprint
                    lane.active = []
                    continue
                ev = torch.cuda.Event()
                ev.record(lane.stream)
                lane.event, lane.chunk = ev, k
                st.chunks += 1
                st.steps += k
                launched = True
            in_flight = sum(len(l.active) for l in self.lanes) + (1 if solo is not None and solo.active else 0)
            st.max_in_flight = max(st.max_in_flight, in_flight)
            st.peak_footprint = max(st.peak_footprint, used)
            if not launched:
                time.sleep(0.0002)
        return results


def run_fifo_plain(requests, device: int = 0, crossover: int = 4096, realtime: bool = True,
                   keep_results: bool = True, clock=time.perf_counter, timing: bool = False,
                   stream_ptr: int | None = None):
    """The single-system solver serving the requests one at a time, in arrival
    order. With timing=True each Result carries the phases of its service
    (host clock, with the stream synchronised at each boundary): `setup`
    (context creation and the initial state), `steps`, `download`, `teardown`
    (context destruction), and `stages`, the library's per-stage device time
    of the steps ({stage: ms}, CUDA events on the context's stream)."""
    pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
    results: dict[int, Result] = {}
    t0 = clock()
    now = lambda: clock() - t0  # noqa: E731
    for req in pending:
        if realtime:
            wait = req.arrival - now()
            if wait > 0:
                time.sleep(wait)
        start = now()
        mode = "pp" if req.n < crossover else "bh"
        tm = {} if timing else None
        try:
            s = ParticleSolverCUDA(req.dt, req.eps2, req.n, mode=mode, theta2=req.theta2, device=device)
            if stream_ptr is not None:
                s.set_stream(stream_ptr)
            try:
                if req.init == "state":
                    s.upload(req.state)
                else:
                    s.init_device(req.init, seed=req.seed, params=req.params)
                if timing:
                    s.sync()
                    tm["setup"] = now() - start
                    s.profile_enable(True)
                    t1 = now()
                s.step(req.steps)
                if timing:
                    s.sync()
                    tm["steps"] = now() - t1
                    tm["stages"] = {k: v[0] for k, v in s.profile_read().items()}
                    s.profile_enable(False)
                    t1 = now()
                out = None
                if keep_results:
                    z = np.zeros((req.n, 4), np.float32)
                    out = ParticleSystem(z, z.copy(), np.zeros(req.n, np.float32), z.copy())
                    s.download(out, masses=True)
                else:
                    s.sync()
                if timing:
                    tm["download"] = now() - t1
                    t1 = now()
            finally:
                s.close()
            if timing:
                tm["teardown"] = now() - t1
            results[req.rid] = Result(req.rid, True, mode, out, arrival=req.arrival, admitted=start,
                                      completed=now(), timing=tm)
        except NBodyError as e:
            results[req.rid] = Result(req.rid, False, mode, error=str(e), arrival=req.arrival, admitted=start,
                                      completed=now(), timing=tm)
    return results


def fifo_replay(requests, service_s: dict) -> dict:
    """Completion times of a one-at-a-time FIFO server for this arrival trace,
    given each request's service time (seconds, by rid): a request starts when
    it has arrived and its predecessor has finished. The service of the plain
    solver does not depend on when a request arrived, so service times measured
    on one trace give the FIFO latencies of the same requests on another."""
    out: dict[int, Result] = {}
    free = 0.0
    for req in sorted(requests, key=lambda r: (r.arrival, r.rid)):
        start = max(free, req.arrival)
        free = start + float(service_s[req.rid])
        out[req.rid] = Result(req.rid, True, arrival=req.arrival, admitted=start, completed=free)
    return out


def poisson_trace(count: int, rate: float, seed: int = 11, n_lo: int = 1024, n_hi: int = 4_194_304,
                  steps_lo: int = 10, steps_hi: int = 500):
    """Requests of the serving workload: Poisson arrivals at `rate` per second;
    a Plummer sphere (a = 100) or a uniform ball (R = 100), N log-uniform in
    [n_lo, n_hi], steps uniform in [steps_lo, steps_hi], dt in {0.001,
    0.0035}, eps^2 uniform in [10, 40], theta = 0.5."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    out = []
    for i in range(count):
        n = int(min(n_hi, np.floor(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi + 1))))))
        kind = "plummer" if rng.random() < 0.5 else "uniform_ball"
        params = (100.0, 1.0, 20.0) if kind == "plummer" else (100.0, 1.0, 10.0)
        out.append(Request(rid=i, n=n, steps=int(rng.integers(steps_lo, steps_hi + 1)),
                           dt=float(rng.choice([0.001, 0.0035])), eps2=float(rng.uniform(10.0, 40.0)), theta2=0.25,
                           init=kind, params=params, seed=1000 + i, arrival=float(t[i])))
    return out


def summarize(results, requests) -> dict:
    ok = [r for r in results.values() if r.ok]
    lat = [r.latency for r in ok]
    first = min(r.arrival for r in requests)
    last = max((r.completed for r in results.values()), default=first)
    span = max(1e-9, last - first)
    return {"requests": len(requests), "completed": len(ok), "failed": len(results) - len(ok),
            "sims_per_s": len(ok) / span, "makespan_s": round(span, 3),
            "p50_latency_s": round(percentile(lat, 50), 4), "p99_latency_s": round(percentile(lat, 99), 4),
            "mean_latency_s": round(float(np.mean(lat)) if lat else float("nan"), 4)}
