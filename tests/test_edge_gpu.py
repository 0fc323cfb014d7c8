"""Edge inputs the reference accepts: massless test particles (m = 0: they
feel forces and exert none; a cell of massless bodies has no centre of mass
and adds nothing) and an unsoftened potential (eps^2 = 0, the guarded kernels:
a pair at zero distance is skipped as the reference skips j == i). Compared
with the C restatement of -v 2 / -v 6 (oracle/nbody_oracle.c).
"""
import numpy as np
import pytest

from test_bh_gpu import bh_forces, check_large

pytestmark = pytest.mark.gpu


def _rms(got, ref):
    g = np.asarray(got, np.float64)[:, :3]
    r = np.asarray(ref, np.float64)[:, :3]
    e = np.linalg.norm(g - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-30)
    return float(np.sqrt(np.mean(e * e))), float(e.max())


def _massless(n, seed):
    from nbody_gb300 import initializers as I

    pos, vel, mass = I.plummer(n, seed=seed)
    mass = mass.copy()
    mass[np.random.default_rng(seed).random(n) < 0.25] = 0.0
    return pos, vel, mass


def test_pp_massless_particles(nb, cuda, oracle):
    n = 3000
    pos, vel, mass = _massless(n, 81)
    sysm = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="pp").update_particle_positions(sysm)
    rms, mx = _rms(sysm.forces, oracle.pp_forces(pos, mass, 40.0))
    assert rms <= 1e-5 and mx <= 1e-3, (rms, mx)


def test_bh_massless_particles(nb, cuda, oracle):
    torch = cuda
    n = 20_000
    pos, vel, mass = _massless(n, 82)
    f, _ = bh_forces(nb, torch, pos, mass)
    pf = oracle.bh_run(pos, vel, np.zeros_like(pos), mass, 0.0035, 40.0, 1, theta2=0.25, patched=True)[3]
    check_large(f, pf)
    assert np.all(np.isfinite(f))


def test_pp_unsoftened(nb, cuda, oracle):
    from nbody_gb300 import initializers as I

    n = 2000
    pos, vel, mass = I.uniform_ball(n, seed=83)
    sysm = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    nb.ParticleSolverCUDA(0.0035, 0.0, n, mode="pp").update_particle_positions(sysm)
    rms, mx = _rms(sysm.forces, oracle.pp_forces(pos, mass, 0.0))
    assert rms <= 1e-5 and mx <= 1e-3, (rms, mx)


def test_bh_unsoftened(nb, cuda, oracle):
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 20_000
    pos, vel, mass = I.plummer(n, seed=84)
    f, _ = bh_forces(nb, torch, pos, mass, eps2=0.0)
    pf = oracle.bh_run(pos, vel, np.zeros_like(pos), mass, 0.0035, 0.0, 1, theta2=0.25, patched=True)[3]
    assert np.all(np.isfinite(f))
    check_large(f, pf)
