"""FP64 conservation diagnostics on the GPU vs the FP64 oracle
(oracle/nbody_oracle.c: orc_diagnostics_f64, direct pair sum).

Kinetic energy and momenta are FP64 sums of the same FP32 inputs: relative
agreement 1e-10 (summation order only). The potential is accumulated per body
in FP32 (direct sum: relative 1e-5; Barnes-Hut walk at theta = 0.5: 3e-3, the
method's error) and reduced in FP64.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("mode", ["pp", "bh"])
def test_diagnostics_match_fp64_oracle(nb, cuda, oracle, mode):
    from nbody_gb300 import initializers as I

    n = 4096 if mode == "pp" else 50_000
    pos, vel, mass = I.plummer(n, seed=71)
    s = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode=mode)
    s.upload(nb.ParticleSystem(pos.copy(), vel.copy(), mass))
    d = s.diagnostics()
    ref = oracle.diagnostics_f64(pos, vel, mass, 40.0)
    assert d["kinetic"] == pytest.approx(ref[0], rel=1e-10)
    assert _rel(d["momentum"], ref[2:5]) < 1e-9
    assert _rel(d["angular_momentum"], ref[5:8]) < 1e-9
    tol = 1e-5 if mode == "pp" else 3e-3
    assert d["potential"] == pytest.approx(ref[1], rel=tol)


def test_diagnostics_follow_resident_bh_state(nb, cuda, oracle):
    """After Barnes-Hut steps the state is in key order; diagnostics see the same system."""
    from nbody_gb300 import initializers as I

    n = 20_000
    pos, vel, mass = I.plummer(n, seed=72)
    system = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    s = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="bh")
    s.upload(system)
    s.step(3)
    d = s.diagnostics()
    s.download(system)
    ref = oracle.diagnostics_f64(system.positions, system.velocities, mass, 40.0)
    assert d["kinetic"] == pytest.approx(ref[0], rel=1e-10)
    assert _rel(d["angular_momentum"], ref[5:8]) < 1e-9
    assert d["potential"] == pytest.approx(ref[1], rel=3e-3)


def test_direct_sum_conserves_momentum_and_energy(nb, cuda):
    """200 direct-sum steps of a virialised Plummer sphere: momentum stays at
    its FP32 rounding level, total energy within 1e-3."""
    from nbody_gb300 import initializers as I

    n = 4096
    pos, vel, mass = I.plummer(n, a=100.0, seed=73)
    s = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="pp")
    s.upload(nb.ParticleSystem(pos.copy(), vel.copy(), mass))
    d0 = s.diagnostics()
    s.step(200)
    d1 = s.diagnostics()
    p_scale = float(np.sum(mass * np.linalg.norm(vel[:, :3], axis=1)))
    assert np.max(np.abs(np.array(d1["momentum"]) - np.array(d0["momentum"]))) < 1e-5 * p_scale
    assert abs(d1["energy"] - d0["energy"]) < 1e-3 * abs(d0["energy"])
