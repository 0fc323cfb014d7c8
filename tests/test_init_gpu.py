"""Device-side seeded initial conditions (nbody_init_device).

The reference's initialisers (src/ParticleSystemInitializer/*) seed from the
clock or std::random_device, so no run of theirs can be repeated or compared
bit for bit; the checks are (1) the counter-based generator itself, restated in
numpy below and compared bit for bit on the cube kind, (2) reproducibility per
(kind, seed), (3) the geometric and mass properties each reference initialiser
guarantees, and (4) that a device-initialised context steps exactly like one
uploaded from the same arrays.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(z):
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _u01(seed, i, k):
    """Draw k of bodies i: the device generator restated (splitmix64 output function)."""
    with np.errstate(over="ignore"):
        inner = _mix64(i.astype(np.uint64) * np.uint64(0xD1B54A32D192ED03) + np.uint64(k))
        h = _mix64(np.uint64(seed) ^ inner)
    return (h >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def _uab(seed, i, k, a, b):
    a, b = np.float32(a), np.float32(b)
    return a + (b - a) * _u01(seed, i, k)


def _state(nb, n, kind, seed, params=None, mode="pp"):
    s = nb.ParticleSolverCUDA(0.001, 0.0935, n, mode=mode)
    s.init_device(kind, seed=seed, params=params)
    z = np.zeros((n, 4), np.float32)
    sysm = nb.ParticleSystem(z, z.copy(), np.zeros(n, np.float32))
    s.download(sysm, masses=True)
    return s, sysm


def test_cube_matches_numpy_generator(nb, cuda):
    """ParticleSystemCubeInitializer.cpp:15-27 restated: bit-exact against numpy."""
    n, seed = 10_001, 987654321
    _, sysm = _state(nb, n, "cube", seed)
    i = np.arange(n, dtype=np.int64)
    W = np.float32(5.0)
    l = np.float32(np.sqrt(np.float32(75.0))) / np.float32(20.0)
    exp_x = np.stack([_uab(seed, i, k, 0.0, W) for k in range(3)], axis=1)
    exp_v = np.stack([_uab(seed, i, 3 + k, -l, l) for k in range(3)], axis=1)
    exp_m = (np.float32(125.0) / np.float32(n)) * np.float32(1.2) * _uab(seed, i, 6, 0.8, 1.3)
    np.testing.assert_array_equal(sysm.positions[:, :3], exp_x)
    np.testing.assert_array_equal(sysm.velocities[:, :3], exp_v)
    np.testing.assert_array_equal(sysm.masses[:, 0], exp_m)
    assert np.all(sysm.positions[:, 3] == 0) and np.all(sysm.accelerations == 0)


KINDS = ["cube", "galaxy", "sphere", "ball", "cube_surface", "plummer", "uniform_ball", "two_discs"]


@pytest.mark.parametrize("kind", KINDS)
def test_same_seed_same_bits(nb, cuda, kind):
    n = 4096
    _, a = _state(nb, n, kind, 11)
    _, b = _state(nb, n, kind, 11, mode="bh")
    _, c = _state(nb, n, kind, 12)
    for x, y in ((a.positions, b.positions), (a.velocities, b.velocities), (a.masses, b.masses)):
        np.testing.assert_array_equal(x, y)
    assert np.all(np.isfinite(a.positions)) and np.all(np.isfinite(a.velocities))
    assert np.all(a.masses[:, 0] > 0)
    assert not np.array_equal(a.positions, c.positions)


def _world():
    return np.array([5.0, 5.0, 5.0]), np.array([2.5, 2.5, 2.5]), float(np.sqrt(75.0))


@pytest.mark.parametrize("pattern", [0, 1, 2])
def test_sphere_surface(nb, cuda, pattern):
    """ParticleSystemSphere.cpp:20-95: |x - c| = |W| / 3; speed in [0.5, 1.5) |W| / 15,
    radial out / in, or along axis x (x - c)."""
    n = 20_000
    W, C, wl = _world()
    _, s = _state(nb, n, "sphere", 5, params=[5, 5, 5, pattern])
    d = s.positions[:, :3].astype(np.float64) - C
    r = np.linalg.norm(d, axis=1)
    np.testing.assert_allclose(r, wl / 3, rtol=2e-6)
    v = s.velocities[:, :3].astype(np.float64)
    speed = np.linalg.norm(v, axis=1)
    base = wl / 15
    assert speed.min() >= 0.5 * base * (1 - 1e-5) and speed.max() < 1.5 * base * (1 + 1e-5)
    u = d / r[:, None]
    if pattern == 2:
        ax = np.array([0.2, 1.0, -0.1]) / np.linalg.norm([0.2, 1.0, -0.1])
        t = np.cross(ax, d)
        ok = np.linalg.norm(t, axis=1) > 1e-3
        np.testing.assert_allclose(np.sum(v[ok] * u[ok], axis=1), 0, atol=1e-5 * base)
        np.testing.assert_allclose(v[ok] @ ax, 0, atol=1e-5 * base)
    else:
        cosang = np.sum(v * u, axis=1) / speed
        np.testing.assert_allclose(cosang, 1.0 if pattern == 0 else -1.0, atol=1e-5)
    # isotropic: the mean direction is near zero
    assert np.linalg.norm(u.mean(axis=0)) < 0.03
    avg = 125.0 / n * 0.5
    m = s.masses[:, 0]
    assert m.min() >= 0.7 * avg * (1 - 1e-5) and m.max() < 1.3 * avg * (1 + 1e-5)


def test_ball(nb, cuda):
    """ParticleSystemBall.cpp:19-75: inside |W|/3 (+5% nudges per axis), uniform in
    volume, masses in [avg/2, 5 avg] skewed low (mean avg/2 + 4.5 avg / 3)."""
    n = 50_000
    W, C, wl = _world()
    _, s = _state(nb, n, "ball", 6)
    R = wl / 3
    d = s.positions[:, :3].astype(np.float64) - C
    r = np.linalg.norm(d, axis=1)
    assert r.max() <= R + 0.05 * R * np.sqrt(3) + 1e-5
    # uniform in volume: fraction inside R/2 ~ 1/8 (nudges blur it slightly)
    assert abs(np.mean(r < R / 2) - 0.125) < 0.01
    v = s.velocities[:, :3]
    assert np.abs(v).max() <= wl * 0.001 * (1 + 1e-5)
    avg = 125.0 / n
    m = s.masses[:, 0].astype(np.float64)
    assert m.min() >= 0.5 * avg * (1 - 1e-5) and m.max() <= 5 * avg * (1 + 1e-5)
    assert m.mean() == pytest.approx(0.5 * avg + 4.5 * avg / 3, rel=0.02)


def test_cube_surface(nb, cuda):
    """ParticleSystemCubeSurface.cpp:15-50: every body on a face of [0, 5]^3, faces equally likely."""
    n = 60_000
    _, s = _state(nb, n, "cube_surface", 7)
    x = s.positions[:, :3]
    on = (x == 0.0) | (x == 5.0)
    assert np.all(on.sum(axis=1) >= 1)
    assert np.all((x >= 0) & (x <= 5))
    faces = np.stack([x[:, 0] == 0, x[:, 0] == 5, x[:, 1] == 0, x[:, 1] == 5, x[:, 2] == 0, x[:, 2] == 5])
    frac = faces.mean(axis=1)
    np.testing.assert_allclose(frac, 1 / 6, atol=0.01)


def test_galaxy(nb, cuda):
    """ParticleSystemGalaxyInitializer.cpp:46-90 (fixed-shape branch): radius < W.x,
    height in [0.1, W.z / 5) above the centre plane, bulge mass 0.7, disc 0.5
    (x volume / n), speeds of order |W| / 4."""
    n = 30_000
    W, C, wl = _world()
    _, s = _state(nb, n, "galaxy", 8)
    d = s.positions[:, :3].astype(np.float64) - C
    R = np.linalg.norm(d[:, :2], axis=1)
    assert R.max() < 5.0 + 1e-4
    assert d[:, 2].min() >= 0.1 - 1e-6 and d[:, 2].max() < 1.0 + 1e-6
    m = s.masses[:, 0]
    unit = 125.0 / n
    bulge = R < 0.5 - 1e-4
    disc = R > 0.5 + 1e-4
    np.testing.assert_allclose(m[bulge], 0.7 * unit, rtol=1e-6)
    np.testing.assert_allclose(m[disc], 0.5 * unit, rtol=1e-6)
    v = s.velocities[:, :3]
    assert np.all(v[:, 2] == 0)
    sp = np.linalg.norm(v, axis=1)
    assert sp.max() <= 2 * wl / 4 * (1 + 1e-5)
    # outside the arm radius the velocity is the pure tangential |W| / 4
    out = R > 2.5 + 1e-3
    np.testing.assert_allclose(sp[out], wl / 4, rtol=1e-5)


def test_plummer_profile_and_virial(nb, cuda):
    """Plummer sphere: half-mass radius a / sqrt(2^(2/3) - 1) = 1.305 a; virial
    ratio 2K / |U| near 1 (direct-sum potential, eps small against a)."""
    n, a = 16_384, 100.0
    s, st = _state(nb, n, "plummer", 9, params=[a, 1.0, 20.0])
    r = np.linalg.norm(st.positions[:, :3].astype(np.float64), axis=1)
    assert np.median(r) == pytest.approx(a / np.sqrt(2 ** (2 / 3) - 1), rel=0.03)
    assert r.max() <= 20 * a * (1 + 1e-6)
    d = s.diagnostics()
    assert 2 * d["kinetic"] / abs(d["potential"]) == pytest.approx(1.0, abs=0.06)
    np.testing.assert_array_equal(st.masses[:, 0], 1.0)


def test_uniform_ball(nb, cuda):
    n = 20_000
    _, s = _state(nb, n, "uniform_ball", 10, params=[100.0, 1.0, 10.0])
    r = np.linalg.norm(s.positions[:, :3].astype(np.float64), axis=1)
    assert r.max() <= 100.0 * (1 + 1e-6)
    assert abs(np.mean(r < 50.0) - 0.125) < 0.01
    m = s.masses[:, 0]
    assert m.min() >= 1.0 and m.max() <= 10.0
    assert np.all(s.velocities == 0)


def test_two_discs(nb, cuda):
    """Central masses first in each half, at -+ separation / 2; star circular
    velocities perpendicular to the in-plane radius of their disc."""
    n = 40_000
    p = [200.0, 20.0, 1e6, 2000.0, 50.0, 30.0, 40.0, 1.0]
    _, s = _state(nb, n, "two_discs", 13, params=p)
    x, v, m = s.positions[:, :3].astype(np.float64), s.velocities[:, :3].astype(np.float64), s.masses[:, 0]
    h = n // 2
    np.testing.assert_allclose(x[0], [-1000.0, 0, 0], atol=1e-3)
    np.testing.assert_allclose(x[h], [1000.0, 0, 0], atol=1e-3)
    np.testing.assert_allclose(v[0], [0, -25.0, 0], atol=1e-4)
    np.testing.assert_allclose(v[h], [0, 25.0, 0], atol=1e-4)
    assert m[0] == m[h] == np.float32(1e6)
    stars = np.r_[1:h]
    d = x[stars] - x[0]
    vr = v[stars] - v[0]
    np.testing.assert_allclose(np.sum(d[:, :2] * vr[:, :2], axis=1) / np.linalg.norm(d[:, :2], axis=1), 0,
                               atol=1e-3 * np.abs(vr).max())
    # exponential surface density: mean radius 2 Rd
    assert np.mean(np.linalg.norm(d[:, :2], axis=1)) == pytest.approx(2 * 200.0, rel=0.02)


@pytest.mark.parametrize("mode", ["pp", "bh"])
def test_device_init_steps_like_upload(nb, cuda, mode):
    """A device-initialised context and one uploaded from the same arrays give
    the same state after steps, bit for bit."""
    n = 8192
    a, st = _state(nb, n, "plummer", 21, mode=mode)
    b = nb.ParticleSolverCUDA(0.001, 0.0935, n, mode=mode)
    b.upload(nb.ParticleSystem(st.positions.copy(), st.velocities.copy(), st.masses[:, 0].copy()))
    a.step(3)
    b.step(3)
    z = np.zeros((n, 4), np.float32)
    ra = nb.ParticleSystem(z.copy(), z.copy(), np.zeros(n, np.float32))
    rb = nb.ParticleSystem(z.copy(), z.copy(), np.zeros(n, np.float32))
    a.download(ra, masses=True)
    b.download(rb, masses=True)
    np.testing.assert_array_equal(ra.masses, rb.masses)
    np.testing.assert_array_equal(ra.positions, rb.positions)
    np.testing.assert_array_equal(ra.velocities, rb.velocities)


def test_init_device_rejects_bad_arguments(nb, cuda):
    s = nb.ParticleSolverCUDA(0.001, 0.0935, 101, mode="pp")
    for kind, params in ((3, None), (99, None), ("cube", [1.0] * 9), ("two_discs", None)):
        with pytest.raises(nb.NBodyError):
            s.init_device(kind, seed=1, params=params)
