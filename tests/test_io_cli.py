"""Particle-file formats, the restated Lagrange initialiser and the headless
command line, checked against the reference's own outputs. No GPU needed."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden


def test_text_writer_matches_reference_writer(nb, tmp_path):
    from nbody_gb300 import io

    g = golden("system_4.npz")
    system = nb.ParticleSystem(g["pos"], g["vel"], g["mass"], g["acc"])
    out = tmp_path / "s.txt"
    io.write_text(system, str(out))
    assert out.read_text() == open(os.path.join(GOLDEN, "system_4.txt")).read()


def test_text_reader_reads_reference_dump(nb):
    from nbody_gb300 import io

    g = golden("system_4.npz")
    s = io.read_text(os.path.join(GOLDEN, "system_4.txt"))
    assert s.n == 4
    # 6 significant digits, as the reference writes them
    np.testing.assert_allclose(s.positions[:, :3], g["pos"][:, :3], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(s.velocities[:, :3], g["vel"][:, :3], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(s.accelerations[:, :3], g["acc"][:, :3], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(s.masses[:, 0], g["mass"], rtol=1e-5)
    assert np.all(s.positions[:, 3] == 0)


def test_text_reader_agrees_with_reference_reader(nb, oracle):
    if not oracle.ref_available():
        pytest.skip("reference build absent")
    import ctypes

    from nbody_gb300 import io

    path = os.path.join(GOLDEN, "system_4.txt")
    s = io.read_text(path)
    p, v, a = (np.zeros((4, 4), np.float32) for _ in range(3))
    m = np.zeros(4, np.float32)
    f = ctypes.POINTER(ctypes.c_float)
    n = oracle.ref().ref_load_text(path.encode(), 4, p.ctypes.data_as(f), v.ctypes.data_as(f), a.ctypes.data_as(f),
                                   m.ctypes.data_as(f))
    assert n == 4
    np.testing.assert_array_equal(s.positions, p)
    np.testing.assert_array_equal(s.velocities[:, :3], v[:, :3])
    np.testing.assert_array_equal(s.accelerations[:, :3], a[:, :3])
    np.testing.assert_array_equal(s.masses[:, 0], m)


def test_binary_round_trip_is_lossless(nb, tmp_path):
    from nbody_gb300 import initializers as I
    from nbody_gb300 import io

    pos, vel, mass = I.plummer(1000, seed=3)
    acc = np.random.default_rng(1).normal(size=(1000, 4)).astype(np.float32)
    s = nb.ParticleSystem(pos, vel, mass, acc)
    io.save_binary(s, str(tmp_path / "s.bin"))
    t = io.load_binary(str(tmp_path / "s.bin"))
    for x, y in ((s.positions, t.positions), (s.velocities, t.velocities), (s.accelerations, t.accelerations),
                 (s.masses, t.masses)):
        np.testing.assert_array_equal(x, y)


def test_lagrange_initialiser_matches_reference():
    from nbody_gb300 import initializers as I

    g = golden("lagrange.npz")
    pos, vel, mass = I.lagrange((5.0, 5.0, 5.0))
    np.testing.assert_allclose(pos, g["pos"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(vel, g["vel"], rtol=1e-6, atol=1e-7)
    np.testing.assert_array_equal(mass, g["mass"])


@pytest.mark.parametrize("argv,msg", [(["-v", "7"], "Invalid version"), (["-v", "8", "-n", "0"],
                                                                         "Invalid number of particles"),
                                       (["-v", "8", "-i", "8"], "Invalid initialization type")])
def test_cli_rejects_bad_arguments(argv, msg):
    r = subprocess.run([sys.executable, "-m", "nbody_gb300", *argv], capture_output=True, text=True,
                       cwd=os.path.join(ROOT, "n-body_gb300"))
    assert r.returncode == 1
    assert msg in r.stderr
