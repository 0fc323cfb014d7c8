"""Seeded synthetic initial conditions for the benchmark and test workloads.

The reference seeds its initialisers from std::random_device or the clock
(e.g. src/ParticleSystemInitializer/ParticleSystemBall/ParticleSystemBall.cpp:15-16),
so its runs cannot be repeated; these generators take an explicit seed
(numpy PCG64) and return the reference's host layout: float32 (n, 4) position
and velocity vec4 arrays (w = 0) and float32 (n,) masses. G = 1 throughout.

* ``uniform_ball``  -- positions uniform in a ball, masses U[lo, hi), v = 0
  (the direct-sum workload: N = 16,384, R = 100, m ~ U[1, 10)).
* ``plummer``       -- equal-mass Plummer sphere, r = a / sqrt(u^(-2/3) - 1)
  truncated at ``rmax`` (20 a), isotropic directions, speeds drawn from the
  Plummer distribution function by rejection sampling (the Barnes-Hut
  workload: N = 2^20, a = 100).
* ``two_discs``     -- two exponential discs (scale length, sech^2 height),
  each with a central point mass, on an inclined encounter (the Barnes-Hut
  scale workload: N = 2^24).
"""
from __future__ import annotations

import numpy as np


def _vec4(xyz: np.ndarray) -> np.ndarray:
    out = np.zeros((xyz.shape[0], 4), np.float32)
    out[:, :3] = xyz
    return out


def _isotropic(rng: np.random.Generator, n: int) -> np.ndarray:
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return d


def uniform_ball(n: int, radius: float = 100.0, mass_range=(1.0, 10.0), seed: int = 12345):
    rng = np.random.default_rng(seed)
    r = radius * rng.random(n) ** (1.0 / 3.0)
    pos = _vec4(r[:, None] * _isotropic(rng, n))
    vel = np.zeros((n, 4), np.float32)
    mass = rng.uniform(mass_range[0], mass_range[1], n).astype(np.float32)
    return pos, vel, mass


def plummer(n: int, a: float = 100.0, mass: float = 1.0, rmax_over_a: float = 20.0, seed: int = 12345, G: float = 1.0):
    rng = np.random.default_rng(seed)
    # radii by inverse transform of M(<r)/M = r^3 / (r^2 + a^2)^1.5, truncated at rmax
    r = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        u = rng.random(todo.size)
        u = np.clip(u, 1e-12, None)
        rr = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        ok = rr <= rmax_over_a * a
        r[todo[ok]] = rr[ok]
        todo = todo[~ok]
    pos = r[:, None] * _isotropic(rng, n)
    # speeds: q = v / v_esc with density g(q) = q^2 (1 - q^2)^3.5 (max < 0.1), rejection sampled
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        x = rng.random(todo.size)
        y = 0.1 * rng.random(todo.size)
        ok = y < x * x * (1.0 - x * x) ** 3.5
        q[todo[ok]] = x[ok]
        todo = todo[~ok]
    total_mass = n * mass
    v_esc = np.sqrt(2.0 * G * total_mass / np.sqrt(r * r + a * a))
    vel = (q * v_esc)[:, None] * _isotropic(rng, n)
    # remove the bulk motion so that the cluster is at rest at the origin
    pos -= pos.mean(axis=0)
    vel -= vel.mean(axis=0)
    return _vec4(pos), _vec4(vel), np.full(n, mass, np.float32)


def exponential_disc(rng: np.random.Generator, n_stars: int, scale_length: float, scale_height: float,
                     central_mass: float, star_mass: float = 1.0, eps2: float = 40.0, G: float = 1.0):
    """One disc in its own frame (z = spin axis), centre mass first."""
    R = rng.gamma(2.0, scale_length, n_stars)              # Sigma ~ exp(-R/Rd) => p(R) ~ R exp(-R/Rd)
    phi = rng.random(n_stars) * 2.0 * np.pi
    z = scale_height * np.arctanh(np.clip(2.0 * rng.random(n_stars) - 1.0, -0.999999, 0.999999))
    order = np.argsort(R)
    enclosed = np.empty(n_stars)
    enclosed[order] = central_mass + star_mass * np.arange(n_stars)
    vc = np.sqrt(G * enclosed * R * R / (R * R + eps2) ** 1.5)
    pos = np.stack([R * np.cos(phi), R * np.sin(phi), z], axis=1)
    vel = np.stack([-vc * np.sin(phi), vc * np.cos(phi), np.zeros(n_stars)], axis=1)
    pos = np.concatenate([np.zeros((1, 3)), pos])
    vel = np.concatenate([np.zeros((1, 3)), vel])
    mass = np.concatenate([[central_mass], np.full(n_stars, star_mass)])
    return pos, vel, mass


def two_discs(n_per_disc_stars: int = 8_388_607, scale_length: float = 200.0, scale_height: float = 20.0,
              central_mass: float = 1e6, separation: float = 2000.0, rel_speed: float = 50.0,
              inclination_deg: float = 30.0, seed: int = 12345):
    rng = np.random.default_rng(seed)
    p1, v1, m1 = exponential_disc(rng, n_per_disc_stars, scale_length, scale_height, central_mass)
    p2, v2, m2 = exponential_disc(rng, n_per_disc_stars, scale_length, scale_height, central_mass)
    t = np.deg2rad(inclination_deg)
    rot = np.array([[1.0, 0.0, 0.0], [0.0, np.cos(t), -np.sin(t)], [0.0, np.sin(t), np.cos(t)]])
    p2 = p2 @ rot.T
    v2 = v2 @ rot.T
    p1[:, 0] -= separation / 2.0
    p2[:, 0] += separation / 2.0
    v1[:, 1] -= rel_speed / 2.0
    v2[:, 1] += rel_speed / 2.0
    pos = np.concatenate([p1, p2])
    vel = np.concatenate([v1, v2])
    mass = np.concatenate([m1, m2]).astype(np.float32)
    return _vec4(pos), _vec4(vel), mass


def lagrange(world=(5.0, 5.0, 5.0), G: float = 1.0):
    """The reference's one deterministic initialiser (-i 3,
    src/ParticleSystemInitializer/ParticleSystemLagrange/ParticleSystemLagrange.cpp:8-50),
    restated in float32: three bodies of mass 10.5 on an equilateral triangle of
    side |world| / 10 around the world centre, each moving tangentially at half
    the speed sqrt(G M / r) for total mass M and distance r to the centre of mass."""
    f = np.float32
    w = np.asarray(world, np.float32)
    mass = f(10.5)
    side = f(np.sqrt(f(np.dot(w, w)))) / f(10.0)
    s3 = f(np.sqrt(f(3.0)))
    c = w / f(2.0)
    v1 = c + np.array([0.0, side / s3, 0.0], np.float32)
    v2 = c + np.array([-side / f(2.0), -side / (f(2.0) * s3), 0.0], np.float32)
    v3 = c + np.array([side / f(2.0), -side / (f(2.0) * s3), 0.0], np.float32)
    com = (v1 + v2 + v3) / f(3.0)
    total = mass * f(3)
    zhat = np.array([0.0, 0.0, 1.0], np.float32)
    pos = np.zeros((3, 4), np.float32)
    vel = np.zeros((3, 4), np.float32)
    for k, vert in enumerate((v1, v2, v3)):
        d = vert - com
        r = f(np.sqrt(f(np.dot(d, d))))
        speed = f(np.sqrt(f(G) * total / r))
        t = np.cross(d, zhat).astype(np.float32)
        t = t * (f(1.0) / f(np.sqrt(f(np.dot(t, t)))))
        pos[k, :3] = vert
        vel[k, :3] = (t * speed) * f(0.5)
    return pos, vel, np.full(3, mass, np.float32)


def ragged_sizes(count: int = 2048, lo: int = 256, hi: int = 131072, seed: int = 2024) -> np.ndarray:
    """System sizes log-uniform in [lo, hi] (the batched-ensemble workload)."""
    rng = np.random.default_rng(seed)
    return np.minimum(hi, np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), count)))).astype(np.int64)


def pos_mass(pos4: np.ndarray, mass: np.ndarray) -> np.ndarray:
    """Device layout: (x, y, z, m) per body."""
    out = np.array(pos4, dtype=np.float32, copy=True)
    out[:, 3] = mass
    return out
