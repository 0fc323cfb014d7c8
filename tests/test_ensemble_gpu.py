"""Ensembles of independent systems (nbody_ensemble_*).

Barnes-Hut systems in an ensemble reproduce the single-system solver bit for
bit (same keys, same stable order inside the system, same tree, same walk);
direct-sum systems agree with the single-system kernel and with the -v 2 port
(oracle/nbody_oracle.c: orc_pp_run) to FP32 summation-order level. Every system
is the same alone and in any mix, bit for bit, eager or replayed from CUDA
graphs, and across membership changes that move it in memory.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PLUMMER = [50.0, 1.0, 20.0]  # a = 50, m = 1, truncated at 20 a


def _empty(nb, n):
    z = np.zeros((n, 4), np.float32)
    return nb.ParticleSystem(z, z.copy(), np.zeros(n, np.float32), z.copy())


def _single(nb, n, mode, seed, steps, dt=0.0035, eps2=40.0, theta2=0.25, integrator="cpu", keys="octree"):
    s = nb.ParticleSolverCUDA(dt, eps2, n, mode=mode, theta2=theta2)
    s.set_integrator(integrator)
    if mode == "bh":
        s.set_key_mode(keys)
    s.init_device("plummer", seed=seed, params=PLUMMER)
    s.step(steps)
    out = _empty(nb, n)
    s.download(out, masses=True)
    s.close()
    return out


def _same(a, b):
    np.testing.assert_array_equal(a.positions, b.positions)
    np.testing.assert_array_equal(a.velocities, b.velocities)
    np.testing.assert_array_equal(a.accelerations, b.accelerations)
    np.testing.assert_array_equal(a.masses, b.masses)


def test_bh_ensemble_matches_single_solver_bit_for_bit(nb, cuda):
    sizes = [20_000, 3_000, 257, 9_001, 64, 1]
    prm = [(0.0035, 40.0, 0.25), (0.001, 10.0, 0.36), (0.0035, 25.0, 0.25), (0.002, 40.0, 0.16),
           (0.0035, 40.0, 0.25), (0.0035, 40.0, 0.25)]
    with nb.Ensemble(crossover=0) as ens:
        ids = []
        for k, (n, (dt, e2, th)) in enumerate(zip(sizes, prm)):
            sid = ens.add(n, dt, e2, th)
            assert ens.info(sid) == ("bh", n)
            ens.init_device(sid, "plummer", seed=100 + k, params=PLUMMER)
            ids.append(sid)
        ens.step(3)
        for k, (n, (dt, e2, th)) in enumerate(zip(sizes, prm)):
            if n < 2:
                continue
            _same(ens.download(ids[k]), _single(nb, n, "bh", 100 + k, 3, dt, e2, th))


def test_bh_ensemble_gpu_euler_and_morton_keys(nb, cuda):
    n = 5_000
    with nb.Ensemble(crossover=0, key_mode="morton") as ens:
        a = ens.add(n, 0.0035, 40.0, 0.25, integrator="gpu_euler")
        b = ens.add(3_000, 0.0035, 40.0, 0.25)
        ens.init_device(a, "plummer", seed=7, params=PLUMMER)
        ens.init_device(b, "plummer", seed=8, params=PLUMMER)
        ens.step(2)
        _same(ens.download(a), _single(nb, n, "bh", 7, 2, integrator="gpu_euler", keys="morton"))


def test_pp_ensemble_matches_single_kernel_and_port(nb, cuda, oracle):
    sizes = [4_000, 700, 256, 33, 1_500]
    with nb.Ensemble(crossover=1 << 30) as ens:
        ids = []
        for k, n in enumerate(sizes):
            sid = ens.add(n, 0.0035, 40.0)
            assert ens.info(sid) == ("pp", n)
            ens.init_device(sid, "plummer", seed=200 + k, params=PLUMMER)
            ids.append(sid)
        start = {sid: ens.download(sid) for sid in ids}
        ens.step(2)
        for k, n in enumerate(sizes):
            got = ens.download(ids[k])
            single = _single(nb, n, "pp", 200 + k, 2)
            np.testing.assert_array_equal(got.masses, single.masses)
            np.testing.assert_allclose(got.positions, single.positions, rtol=1e-6, atol=1e-4)
            s0 = start[ids[k]]
            p, v, a, _, _ = oracle.pp_run(s0.positions, s0.velocities, s0.accelerations, s0.masses[:, 0], 0.0035,
                                          40.0, 2)
            rel = np.linalg.norm(got.accelerations[:, :3] - a[:, :3], axis=1) / np.linalg.norm(a[:, :3], axis=1)
            assert np.sqrt(np.mean(rel ** 2)) < 1e-5
            np.testing.assert_allclose(got.positions, p, rtol=1e-6, atol=1e-4)


def test_each_system_is_the_same_alone_and_in_a_mix(nb, cuda):
    rng = np.random.default_rng(5)
    probe = [(6_000, "bh"), (900, "pp")]
    alone = []
    for k, (n, mode) in enumerate(probe):
        with nb.Ensemble(crossover=2048) as ens:
            sid = ens.add(n, 0.0035, 40.0, 0.25)
            assert ens.info(sid)[0] == mode
            ens.init_device(sid, "plummer", seed=300 + k, params=PLUMMER)
            ens.step(4)
            alone.append(ens.download(sid))
    with nb.Ensemble(crossover=2048) as ens:
        others = []
        for j in range(30):
            n = int(np.exp(rng.uniform(np.log(64), np.log(20_000))))
            sid = ens.add(n, 0.0035, float(rng.uniform(10, 40)), 0.25)
            ens.init_device(sid, "plummer", seed=1000 + j, params=PLUMMER)
            others.append(sid)
        mine = []
        for k, (n, mode) in enumerate(probe):
            sid = ens.add(n, 0.0035, 40.0, 0.25)
            ens.init_device(sid, "plummer", seed=300 + k, params=PLUMMER)
            mine.append(sid)
        ens.step(4)
        for k in range(len(probe)):
            _same(ens.download(mine[k]), alone[k])


def test_graph_replay_equals_eager(nb, cuda):
    def run(graph_steps):
        with nb.Ensemble(crossover=2048) as ens:
            ids = []
            for k, n in enumerate([5_000, 1_000, 300, 12_000]):
                sid = ens.add(n, 0.0035, 40.0, 0.25)
                ens.init_device(sid, "plummer", seed=400 + k, params=PLUMMER)
                ids.append(sid)
            ens.step(7, graph_steps=graph_steps)
            return [ens.download(s) for s in ids]

    eager, graphed = run(0), run(3)
    for a, b in zip(eager, graphed):
        _same(a, b)


def test_membership_changes_keep_states(nb, cuda):
    """Removing and adding systems moves the others in memory; their
    trajectories continue unchanged."""
    ref = []
    for k, n in enumerate([4_000, 700]):
        with nb.Ensemble(crossover=2048) as ens:
            sid = ens.add(n, 0.0035, 40.0)
            ens.init_device(sid, "plummer", seed=500 + k, params=PLUMMER)
            ens.step(4)
            ref.append(ens.download(sid))
    with nb.Ensemble(crossover=2048) as ens:
        a = ens.add(4_000, 0.0035, 40.0)
        gone = ens.add(8_000, 0.0035, 40.0)
        b = ens.add(700, 0.0035, 40.0)
        for sid, seed in ((a, 500), (gone, 9), (b, 501)):
            ens.init_device(sid, "plummer", seed=seed, params=PLUMMER)
        ens.step(2, graph_steps=2)
        ens.remove(gone)
        new = ens.add(30_000, 0.0035, 40.0)
        ens.init_device(new, "uniform_ball")
        ens.step(2, graph_steps=2)
        _same(ens.download(a), ref[0])
        _same(ens.download(b), ref[1])
        c = ens.counts()
        assert c["systems"] == 3 and c["bh_bodies"] == 34_000 and c["pp_bodies"] == 700


def test_upload_matches_init_device(nb, cuda):
    n = 3_000
    with nb.Ensemble(crossover=0) as ens:
        a = ens.add(n, 0.0035, 40.0)
        b = ens.add(n, 0.0035, 40.0)
        ens.init_device(a, "plummer", seed=61, params=PLUMMER)
        ens.upload(b, ens.download(a))
        ens.step(3)
        _same(ens.download(a), ens.download(b))


def test_ensemble_errors(nb, cuda):
    with nb.Ensemble() as ens:
        sid = ens.add(100, 0.001, 1.0)
        with pytest.raises(nb.NBodyError):
            ens.step(1)  # no state yet
        with pytest.raises(nb.NBodyError):
            ens.add(0, 0.001, 1.0)
        with pytest.raises(nb.NBodyError):
            ens.init_device(sid, 99)
        with pytest.raises(nb.NBodyError):
            ens.remove(sid + 7)
        ens.init_device(sid, "cube")
        ens.step(1)
        ens.remove(sid)
        with pytest.raises(nb.NBodyError):
            ens.download(sid)
        ens.step(1)  # empty ensemble: nothing to do
    assert nb.Ensemble.footprint(1 << 20, "bh") > nb.Ensemble.footprint(1 << 20, "pp") > 0
