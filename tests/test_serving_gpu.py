"""Serving on the GPU: continuous batching gives each request the result it
gets alone. Barnes-Hut requests match the single-system solver bit for bit;
direct-sum requests match it to FP32 summation order (positions to 1e-6
relative, accelerations to RMS 1e-5) and match themselves served alone bit for
bit. The memory budget forces queueing, and several requests are in flight
together.
"""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    for x, y in ((a.positions, b.positions), (a.velocities, b.velocities), (a.accelerations, b.accelerations),
                 (a.masses, b.masses)):
        np.testing.assert_array_equal(x, y)


def _trace(serving):
    return serving.poisson_trace(12, rate=300.0, seed=5, n_lo=200, n_hi=40_000, steps_lo=2, steps_hi=12)


def test_served_results_equal_each_request_alone(nb, cuda):
    from nbody_gb300 import serving

    reqs = _trace(serving)
    fps = [2 * nb.Ensemble.footprint(r.n, "pp" if r.n < 4096 else "bh") for r in reqs]
    budget = int(0.4 * sum(fps))
    assert budget >= max(fps)
    with serving.Server(budget_bytes=budget, crossover=4096, pp_shape="128x2", max_chunk=3) as srv:
        res = srv.run_trace(reqs, realtime=True)
        assert srv.stats.max_in_flight >= 2
        assert srv.stats.peak_footprint <= budget
    plain = serving.run_fifo_plain(reqs, crossover=4096, realtime=False)
    modes = set()
    for r in reqs:
        a, b = res[r.rid], plain[r.rid]
        assert a.ok and b.ok, (a.error, b.error)
        assert a.mode == b.mode
        modes.add(a.mode)
        if a.mode == "bh":
            _same(a.system, b.system)
        else:
            np.testing.assert_array_equal(a.system.masses, b.system.masses)
            np.testing.assert_allclose(a.system.positions, b.system.positions, rtol=1e-6, atol=1e-4)
            ga, gb = a.system.accelerations[:, :3], b.system.accelerations[:, :3]
            rel = np.linalg.norm(ga - gb, axis=1) / np.maximum(np.linalg.norm(gb, axis=1), 1e-30)
            assert np.sqrt(np.mean(rel ** 2)) < 1e-5
    assert modes == {"pp", "bh"}
    # alone in the server: bit for bit, whatever shared the launches before
    for r in reqs[:4]:
        with serving.Server(budget_bytes=budget, crossover=4096, pp_shape="128x2", max_chunk=3) as srv:
            one = srv.run_trace([dataclasses.replace(r, arrival=0.0)], realtime=False)
        _same(one[r.rid].system, res[r.rid].system)


@pytest.mark.parametrize("solo_n", [None, 20_000])
def test_lane_server_results_equal_each_request_alone(nb, cuda, solo_n):
    """Priority lanes (concurrent ensembles on streams of different priority)
    give the same bits as the shared server, request by request; so do the
    largest Barnes-Hut requests run alone in the solo lane (the single-system
    solver), here from 20,000 bodies on."""
    from nbody_gb300 import serving

    reqs = _trace(serving)
    with serving.Server(budget_bytes=1e10, crossover=4096, pp_shape="128x2", max_chunk=3) as srv:
        shared = srv.run_trace(reqs, realtime=False)
    # bounds that spread this small trace over all four lanes
    with serving.LaneServer(budget_bytes=1e10, crossover=4096, pp_shape="128x2", max_chunk=3,
                            bounds=(2e4, 1e5, 2e5), solo_n=solo_n) as srv:
        lanes = srv.run_trace(reqs, realtime=True)
        solo = [r for r in reqs if srv.is_solo(r)]
        used = {srv.lane_of(r) for r in reqs if not srv.is_solo(r)}
        assert len(used) >= 3
    if solo_n is not None:
        assert len(solo) >= 2
    for r in reqs:
        assert lanes[r.rid].ok, lanes[r.rid].error
        _same(lanes[r.rid].system, shared[r.rid].system)


def test_requests_with_explicit_states(nb, cuda):
    from nbody_gb300 import initializers as I
    from nbody_gb300 import serving

    reqs = []
    for i, n in enumerate([3_000, 9_000]):
        pos, vel, mass = I.plummer(n, seed=40 + i)
        reqs.append(serving.Request(rid=i, n=n, steps=5, dt=0.0035, eps2=40.0, init="state",
                                    state=nb.ParticleSystem(pos, vel, mass)))
    with serving.Server(budget_bytes=1e9, crossover=4096, pp_shape="128x2") as srv:
        res = srv.run_trace(reqs, realtime=False)
    plain = serving.run_fifo_plain(reqs, crossover=4096, realtime=False)
    _same(res[1].system, plain[1].system)  # Barnes-Hut
    np.testing.assert_allclose(res[0].system.positions, plain[0].system.positions, rtol=1e-6, atol=1e-4)
