"""Serving loop host logic on the CPU, against a fake ensemble (no GPU): the
request trace, admission by memory footprint in arrival order, chunking that
never runs past the soonest finish, retirement, and failure handling.
"""
import numpy as np
import pytest


class FakeEnsemble:
    """Steps nothing; records what the server asks for."""

    crossover = 1000

    def __init__(self, fail_step_at=None):
        self.systems = {}
        self.next = 0
        self.steps = []
        self.fail_step_at = fail_step_at
        self.log = []

    @staticmethod
    def footprint(n, mode):
        return 100 * n

    def add(self, n, dt, eps2, theta2=0.25, mode=None, integrator="cpu"):
        sid = self.next
        self.next += 1
        self.systems[sid] = {"n": n, "steps": 0, "ready": False}
        self.log.append(("add", sid))
        return sid

    def remove(self, sid):
        del self.systems[sid]
        self.log.append(("remove", sid))

    def info(self, sid):
        n = self.systems[sid]["n"]
        return ("pp" if n < self.crossover else "bh"), n

    def init_device(self, sid, kind, seed=0, params=None):
        from nbody_gb300 import NBodyError

        if kind not in ("plummer", "uniform_ball"):
            raise NBodyError(1, "init_device")
        self.systems[sid]["ready"] = True

    def upload(self, sid, system):
        self.systems[sid]["ready"] = True

    def step(self, k, graph_steps=0):
        from nbody_gb300 import NBodyError

        if self.fail_step_at is not None and len(self.steps) == self.fail_step_at:
            self.steps.append(-k)
            raise NBodyError(5, "nbody_ensemble_step")
        self.steps.append(k)
        for s in self.systems.values():
            assert s["ready"]
            s["steps"] += k

    def sync(self):
        pass

    def download(self, sid):
        return self.systems[sid]["steps"]  # the step count stands in for the state

    def close(self):
        pass


def _req(serving, rid, n, steps, arrival=0.0, init="plummer"):
    return serving.Request(rid=rid, n=n, steps=steps, dt=0.001, eps2=10.0, init=init, arrival=arrival)


def test_trace_statistics():
    from nbody_gb300 import serving

    tr = serving.poisson_trace(4000, rate=100.0, seed=3)
    gaps = np.diff([0.0] + [r.arrival for r in tr])
    assert np.mean(gaps) == pytest.approx(0.01, rel=0.05)
    ns = np.array([r.n for r in tr])
    assert ns.min() >= 1024 and ns.max() <= 4_194_304
    # log-uniform: the median is near the geometric mean of the range
    assert np.median(ns) == pytest.approx(np.sqrt(1024 * 4_194_304), rel=0.15)
    st = np.array([r.steps for r in tr])
    assert st.min() >= 10 and st.max() <= 500
    assert {r.dt for r in tr} == {0.001, 0.0035}
    assert all(10.0 <= r.eps2 <= 40.0 for r in tr)
    assert {r.init for r in tr} == {"plummer", "uniform_ball"}


def test_every_request_gets_exactly_its_steps():
    from nbody_gb300 import serving

    fake = FakeEnsemble()
    reqs = [_req(serving, i, 100 + 37 * i, steps) for i, steps in enumerate([7, 23, 3, 40, 11, 5, 19])]
    with serving.Server(budget_bytes=10**9, crossover=1000, pp_shape="256x2", max_chunk=10, ensemble=fake) as srv:
        res = srv.run_trace(reqs, realtime=False)
    for r in reqs:
        assert res[r.rid].ok and res[r.rid].system == r.steps
    # a chunk never exceeds max_chunk
    assert max(fake.steps) <= 10
    assert not fake.systems  # everything retired


def test_admission_respects_the_budget_in_arrival_order():
    from nbody_gb300 import serving

    fake = FakeEnsemble()
    # footprint = 2 * 100 * n; budget fits two systems of 1000 at once
    reqs = [_req(serving, i, 1000, 5) for i in range(6)]
    budget = 2 * (2 * 100 * 1000)
    with serving.Server(budget_bytes=budget, crossover=1000, pp_shape="256x2", ensemble=fake) as srv:
        res = srv.run_trace(reqs, realtime=False)
        assert srv.stats.max_in_flight == 2
        assert srv.stats.peak_footprint <= budget
    adds = [sid for op, sid in fake.log if op == "add"]
    assert adds == sorted(adds)
    order = sorted(res.values(), key=lambda r: r.completed)
    assert [r.rid for r in order] == sorted(r.rid for r in order)


def test_oversized_and_broken_requests_fail_alone():
    from nbody_gb300 import serving

    fake = FakeEnsemble()
    reqs = [_req(serving, 0, 100, 4), _req(serving, 1, 10**9, 4), _req(serving, 2, 200, 4, init="nonsense"),
            _req(serving, 3, 300, 4)]
    with serving.Server(budget_bytes=10**7, crossover=1000, pp_shape="256x2", ensemble=fake) as srv:
        res = srv.run_trace(reqs, realtime=False)
    assert res[0].ok and res[3].ok
    assert not res[1].ok and "budget" in res[1].error
    assert not res[2].ok
    assert not fake.systems


def test_a_failed_step_fails_the_requests_in_flight_only():
    from nbody_gb300 import serving

    fake = FakeEnsemble(fail_step_at=1)
    reqs = [_req(serving, 0, 100, 20), _req(serving, 1, 100, 20), _req(serving, 2, 100, 5, arrival=0.0)]
    with serving.Server(budget_bytes=2 * (2 * 100 * 100), crossover=1000, pp_shape="256x2", max_chunk=5,
                        ensemble=fake) as srv:
        res = srv.run_trace(reqs, realtime=False)
    # requests 0 and 1 were in flight at the failing chunk; 2 was admitted afterwards
    assert not res[0].ok and not res[1].ok
    assert res[2].ok and res[2].system == 5


def test_summary_percentiles():
    from nbody_gb300 import serving

    reqs = [_req(serving, i, 10, 1, arrival=float(i)) for i in range(100)]
    res = {i: serving.Result(i, True, arrival=float(i), completed=float(i) + 1.0 + i / 100.0) for i in range(100)}
    s = serving.summarize(res, reqs)
    assert s["completed"] == 100 and s["failed"] == 0
    assert s["p50_latency_s"] == pytest.approx(1.495, abs=1e-3)
    assert s["p99_latency_s"] == pytest.approx(1.9801, abs=1e-3)
    assert s["sims_per_s"] == pytest.approx(100 / (99 + 1.99), rel=1e-6)


def test_fifo_replay_is_the_fifo_recurrence():
    """fifo_replay: a request starts at max(its arrival, the previous finish);
    service times carried over from another trace of the same requests."""
    from nbody_gb300 import serving

    reqs = [_req(serving, 0, 10, 1, arrival=0.0), _req(serving, 1, 10, 1, arrival=0.5),
            _req(serving, 2, 10, 1, arrival=5.0), _req(serving, 3, 10, 1, arrival=5.1)]
    service = {0: 2.0, 1: 1.0, 2: 0.5, 3: 0.25}
    res = serving.fifo_replay(reqs, service)
    assert [res[i].admitted for i in range(4)] == [0.0, 2.0, 5.0, 5.5]
    assert [res[i].completed for i in range(4)] == [2.0, 3.0, 5.5, 5.75]
    assert res[1].latency == 2.5
    s = serving.summarize(res, reqs)
    assert s["completed"] == 4 and s["makespan_s"] == 5.75
