"""Generates the golden fixtures in this directory from the REFERENCE'S OWN CPU
solvers (oracle/_ref/libnbody_ref.so, the reference sources compiled headless).

Run here, where the reference checkout exists:  python tests/golden/make_golden.py
The .npz files it writes are committed; tests read them on any machine.

Every fixture stores the inputs (positions, velocities, accelerations, masses
in the reference's host layout), the parameters, and the reference's outputs.
Barnes-Hut fixtures use one OpenMP thread: -v 6 appends bodies to its task
buckets under locks, so only a one-thread run has a fixed insertion order.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "n-body_gb300"))

import pyoracle as O  # noqa: E402
from nbody_gb300 import initializers as I  # noqa: E402


def _state(n, seed, vel_scale=1.0, acc_scale=0.0, radius=100.0):
    pos, vel, mass = I.uniform_ball(n, radius=radius, seed=seed)
    rng = np.random.default_rng(seed + 1)
    vel[:, :3] = vel_scale * rng.normal(size=(n, 3))
    acc = np.zeros((n, 4), np.float32)
    acc[:, :3] = acc_scale * rng.normal(size=(n, 3))
    return pos, vel, acc, mass


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def pp_case(name, n, seed, steps, dt=0.0035, eps2=40.0, vel_scale=1.0, acc_scale=0.5, version=2):
    pos, vel, acc, mass = _state(n, seed, vel_scale, acc_scale)
    p1, v1, a1, f1, _ = O.ref_run(version, pos, vel, acc, mass, dt, eps2, 1)
    pk, vk, ak, fk, _ = O.ref_run(version, pos, vel, acc, mass, dt, eps2, steps)
    save(name, pos=pos, vel=vel, acc=acc, mass=mass, dt=dt, eps2=eps2, steps=steps, version=version,
         pos1=p1, vel1=v1, acc1=a1, force1=f1, posk=pk, velk=vk, acck=ak, forcek=fk)


def bh_case(name, pos, vel, acc, mass, steps, theta2, dt=0.0035, eps2=40.0):
    # -v 6 has fixed per-task capacities (n/2 nodes per subtree, 0.3 n bodies
    # per task, src/Octree/ParallelOctreeCPU.cpp:27,38,50) and no bounds check:
    # an overflow corrupts its pool and can leave its insert loop spinning. The
    # port applies the same capacities and reports the overflow, so every case
    # is checked with it before the reference runs.
    chk = O.bh_run(pos, vel, acc, mass, dt, eps2, steps, theta2=theta2, threads=1)[4]
    assert chk["rc"] == 0, f"{name}: -v 6 capacity would overflow ({chk})"
    p1, v1, a1, f1, i1 = O.ref_run(6, pos, vel, acc, mass, dt, eps2, 1, theta2=theta2, threads=1)
    pk, vk, ak, fk, ik = O.ref_run(6, pos, vel, acc, mass, dt, eps2, steps, theta2=theta2, threads=1)
    assert abs(i1["root_mass"] - float(mass.astype(np.float64).sum())) <= 1e-3 * float(mass.sum()), i1
    save(name, pos=pos, vel=vel, acc=acc, mass=mass, dt=dt, eps2=eps2, steps=steps, theta2=theta2,
         root_mass1=i1["root_mass"], pos1=p1, vel1=v1, acc1=a1, force1=f1, posk=pk, velk=vk, acck=ak, forcek=fk)


def main():
    if not O.ref_available():
        O.build(reference=True)
    only = sys.argv[1:]
    if only:
        globals()[only[0]]()
        return
    # direct sum, -v 2 (ParticleSolverCPUParallel)
    pp_case("pp_ball_1024.npz", 1024, seed=7, steps=10)
    pp_case("pp_ball_1000.npz", 1000, seed=8, steps=5)            # not a multiple of any tile
    for n in (1, 2, 3, 5, 127):
        pp_case(f"pp_small_{n}.npz", n, seed=100 + n, steps=3, eps2=0.5)
    pp_case("pp_eps0_64.npz", 64, seed=9, steps=2, eps2=0.0)       # no softening: self pair skipped
    # the reference's one deterministic initialiser (-i 3) with its default
    # world size (src/main.cpp:27) and default dt / softening (ArgumentsParser.cpp:6-10)
    pos, vel, acc, mass = O.ref_lagrange((5.0, 5.0, 5.0))
    dt, eps2 = 0.001, 0.0935
    p1, v1, a1, f1, _ = O.ref_run(1, pos, vel, acc, mass, dt, eps2, 1)
    pk, vk, ak, fk, _ = O.ref_run(1, pos, vel, acc, mass, dt, eps2, 1000)
    save("lagrange.npz", pos=pos, vel=vel, acc=acc, mass=mass, dt=dt, eps2=eps2, steps=1000,
         pos1=p1, vel1=v1, acc1=a1, force1=f1, posk=pk, velk=vk, acck=ak, forcek=fk)
    # Barnes-Hut, -v 6 (ParticleSolverBHutCPUParallel), one thread
    pos, vel, acc, mass = _state(2048, seed=11, vel_scale=1.0, acc_scale=0.5)
    bh_case("bh_ball_2048.npz", pos, vel, acc, mass, steps=4, theta2=0.25)
    bh_case("bh_ball_2048_theta06.npz", pos, vel, acc, mass, steps=2, theta2=0.36)
    # A Plummer sphere truncated at 3a: concentrated, yet inside -v 6's fixed capacities.
    pos, vel, mass = I.plummer(4096, a=100.0, rmax_over_a=3.0, seed=12)
    bh_case("bh_plummer_4096.npz", pos, vel, np.zeros_like(pos), mass, steps=3, theta2=0.25)
    # text format written by the reference (src/ParticleSystem/ParticleSystem.cpp:205-215)
    pos, vel, acc, mass = _state(4, seed=13, vel_scale=1.0, acc_scale=0.5)
    text = O.ref_dump_text(pos, vel, acc, mass)
    with open(os.path.join(HERE, "system_4.txt"), "w") as f:
        f.write(text)
    save("system_4.npz", pos=pos, vel=vel, acc=acc, mass=mass)


if __name__ == "__main__":
    main()
