"""Failure detection on the GPU without a fault: every device wait is bounded.
A kernel whose wait can never complete (an mbarrier nothing arrives at) gives
up after its limit, reports NBODY_ERR_TIMEOUT in its status word, and the GPU
stays usable for the next solve. Host-side failures (bad arguments, capacity,
failed serving chunks) are covered in the CPU tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_reports(nb, cuda):
    status, waited = nb.selftest_wait(limit_us=50_000)
    assert status == nb.ERR_TIMEOUT
    assert 50.0 <= waited < 2000.0, waited


def test_gpu_usable_after_a_timed_out_wait(nb, cuda, oracle):
    from nbody_gb300 import initializers as I

    for _ in range(2):
        assert nb.selftest_wait(limit_us=10_000)[0] == nb.ERR_TIMEOUT
    n = 2000
    pos, vel, mass = I.uniform_ball(n, seed=9)
    sysm = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="pp").update_particle_positions(sysm)
    ref = oracle.pp_forces(pos, mass, 40.0)
    rel = np.linalg.norm(sysm.forces[:, :3] - ref[:, :3], axis=1) / np.linalg.norm(ref[:, :3], axis=1)
    assert np.sqrt(np.mean(rel ** 2)) < 1e-5


def test_selftest_rejects_bad_limits(nb, cuda):
    for bad in (0, -5, 2_000_000):
        with pytest.raises(nb.NBodyError):
            nb.selftest_wait(limit_us=bad)
