"""Particle-system files: the reference's text format and a lossless binary one.

Text (what the reference writes with operator<<,
src/ParticleSystem/ParticleSystem.cpp:205-215, and reads with -f,
src/ParticleSystemInitializer/ParticleSystemFile/ParticleSystemFile.cpp:10-90)::

    Particle System with N particles:
    Particle ID: i
    Position: (x, y, z)
    Velocity: (x, y, z)
    Acceleration: (x, y, z)
    Mass: m

Numbers use the stream's default formatting (6 significant digits), so a
text round trip is lossy, as in the reference. The binary file keeps every
bit of positions, velocities, the lagged accelerations (the integrator's `a`,
needed to resume exactly) and masses:

    8 bytes  magic b"NBODYGB1"
    8 bytes  body count n (little-endian uint64)
    16 n     positions   float32 (x, y, z, 0)
    16 n     velocities  float32 (x, y, z, w)
    16 n     accelerations float32 (x, y, z, w)
    4 n      masses      float32
"""
from __future__ import annotations

import re

import numpy as np

from . import ParticleSystem

MAGIC = b"NBODYGB1"


def _fmt(x: float) -> str:
    # The reference streams floats with the default precision: printf("%g").
    return "%g" % float(x)


def write_text(system: ParticleSystem, path: str) -> None:
    p, v, a = system.positions, system.velocities, system.accelerations
    m = system.masses[:, 0]
    out = [f"Particle System with {system.n} particles:\n"]
    for i in range(system.n):
        out.append(f"Particle ID: {i}\n")
        out.append(f"Position: ({_fmt(p[i, 0])}, {_fmt(p[i, 1])}, {_fmt(p[i, 2])})\n")
        out.append(f"Velocity: ({_fmt(v[i, 0])}, {_fmt(v[i, 1])}, {_fmt(v[i, 2])})\n")
        out.append(f"Acceleration: ({_fmt(a[i, 0])}, {_fmt(a[i, 1])}, {_fmt(a[i, 2])})\n")
        out.append(f"Mass: {_fmt(m[i])}\n")
    with open(path, "w") as f:
        f.write("".join(out))


_TRIPLE = re.compile(r"\(([^,]*),([^,]*),([^)]*)\)")


def read_text(path: str) -> ParticleSystem:
    """Reads the reference's text format the way its -f reader does: the count
    from the first line, then Position / Velocity / Acceleration lines, each
    body completed by its Mass line; stops after the announced count."""
    with open(path) as f:
        lines = f.read().splitlines()
    if not lines or "Particle System with " not in lines[0]:
        raise ValueError("Invalid file format. Unable to determine total particles.")
    total = int(lines[0].split("with ", 1)[1].split()[0])
    pos, vel, acc, mass = [], [], [], []
    cur = {"p": (0.0, 0.0, 0.0), "v": (0.0, 0.0, 0.0), "a": (0.0, 0.0, 0.0)}
    for line in lines[1:]:
        if "Particle ID" in line:
            continue
        for tag, key in (("Position:", "p"), ("Velocity:", "v"), ("Acceleration:", "a")):
            if tag in line:
                m = _TRIPLE.search(line)
                if not m:
                    raise ValueError(f"malformed line: {line!r}")
                cur[key] = tuple(np.float32(float(t)) for t in m.groups())
        if "Mass:" in line:
            mass.append(np.float32(float(line.split(":", 1)[1])))
            pos.append(cur["p"])
            vel.append(cur["v"])
            acc.append(cur["a"])
            if len(mass) >= total:
                break
    n = len(mass)
    z = np.zeros((n, 1), np.float32)
    to4 = lambda rows: np.concatenate([np.array(rows, np.float32).reshape(n, 3), z], axis=1)  # noqa: E731
    return ParticleSystem(to4(pos), to4(vel), np.array(mass, np.float32), to4(acc))


def save_binary(system: ParticleSystem, path: str) -> None:
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.uint64(system.n).tobytes())
        f.write(np.ascontiguousarray(system.positions, np.float32).tobytes())
        f.write(np.ascontiguousarray(system.velocities, np.float32).tobytes())
        f.write(np.ascontiguousarray(system.accelerations, np.float32).tobytes())
        f.write(np.ascontiguousarray(system.masses[:, 0], np.float32).tobytes())


def load_binary(path: str) -> ParticleSystem:
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError("not an nbody_gb300 binary particle file")
        n = int(np.frombuffer(f.read(8), np.uint64)[0])
        arr = lambda k: np.frombuffer(f.read(4 * k), np.float32)  # noqa: E731
        pos = arr(4 * n).reshape(n, 4).copy()
        vel = arr(4 * n).reshape(n, 4).copy()
        acc = arr(4 * n).reshape(n, 4).copy()
        mass = arr(n).copy()
    return ParticleSystem(pos, vel, mass, acc)
