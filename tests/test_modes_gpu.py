"""GPU checks of the headless run loop, checkpoint/resume and the GLSL
integrator mode."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, golden, rel_err_stats

pytestmark = pytest.mark.gpu


def test_cli_lagrange_reproduces_reference_run(nb, cuda, tmp_path):
    """-v 8 -i 3 with the reference's defaults for 1,000 steps, written in the
    reference's text format, against the reference's own -v 1 run of the same
    system (golden lagrange.npz; text carries 6 significant digits)."""
    from nbody_gb300 import io

    g = golden("lagrange.npz")
    out = tmp_path / "final.txt"
    r = subprocess.run([sys.executable, "-m", "nbody_gb300", "-v", "8", "-i", "3", "-t", "0.001", "-s", "0.0935",
                        "--steps", "1000", "--dump", str(out)], capture_output=True, text=True,
                       cwd=os.path.join(ROOT, "n-body_gb300"), timeout=300)
    assert r.returncode == 0, r.stderr
    assert "1000 steps" in r.stdout
    s = io.read_text(str(out))
    np.testing.assert_allclose(s.positions[:, :3], g["posk"][:, :3], rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(s.velocities[:, :3], g["velk"][:, :3], rtol=1e-3, atol=1e-3)


@pytest.mark.parametrize("mode", ["pp", "bh"])
def test_resume_from_binary_checkpoint_is_exact(nb, cuda, tmp_path, mode):
    from nbody_gb300 import initializers as I
    from nbody_gb300 import io

    n = 5000
    pos, vel, mass = I.plummer(n, seed=81)
    a = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    s = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode=mode)
    s.update_particle_positions(a, steps=10)
    b = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    s.update_particle_positions(b, steps=5)
    io.save_binary(b, str(tmp_path / "ck.bin"))
    c = io.load_binary(str(tmp_path / "ck.bin"))
    s.update_particle_positions(c, steps=5)
    for x, y in ((a.positions, c.positions), (a.velocities, c.velocities), (a.accelerations, c.accelerations)):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("mode", ["pp", "bh"])
def test_gpu_euler_integrator(nb, cuda, oracle, mode):
    """updateParticles.glsl:44-55: v += F dt; x += v dt (one step from the
    oracle's forces, every operation rounded on its own)."""
    from nbody_gb300 import initializers as I

    n = 3000
    pos, vel, mass = I.plummer(n, seed=82)
    s = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode=mode, theta2=1e-12 if mode == "bh" else 0.25)
    s.set_integrator("gpu_euler")
    sysm = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    s.update_particle_positions(sysm)
    F = oracle.pp_forces(pos, mass, 40.0)
    rms, mx = rel_err_stats(sysm.forces, F)
    assert rms < 1e-5
    f = np.float32
    v = (vel[:, :3] + F[:, :3] * f(0.0035)).astype(np.float32)
    x = (pos[:, :3] + v * f(0.0035)).astype(np.float32)
    np.testing.assert_allclose(sysm.velocities[:, :3], v, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(sysm.positions[:, :3], x, rtol=1e-6, atol=1e-6)
