"""Headless run loop: python -m nbody_gb300 [-v version] [-n numParticles] [-i init]
[-t timeStep] [-s squaredSoftening] [-f filePath] [--steps K] ...

Mirrors the reference's command line (src/ArgumentsParser/ArgumentsParser.cpp:49-106,
long forms -version/-init/-time-step/-softening/-file) with the GPU solver
registered as two new versions, and replaces its window and render loop
(src/RenderLoop/RenderLoop.cpp:12-35) by a fixed number of steps:

  -v 8   direct sum on the GPU   (-v 2 semantics: ParticleSolverCPUParallel)
  -v 9   Barnes-Hut on the GPU   (-v 6 semantics: ParticleSolverBHutCPUParallel)

Versions 1-7 are the reference's own CPU and OpenGL solvers and are not part of
this program. Initialisers (the reference's -i numbers, include/enums.h:3-11):
-i 1 cube, 2 galaxy, 4 sphere surface, 5 ball, 6 cube surface (generated on
the GPU from --seed, in the reference's 5 x 5 x 5 world), -i 3 the Lagrange
triangle, -f FILE (the reference's text format, or this library's lossless
binary format), and -i plummer / discs for the benchmark workloads (also
generated on the GPU). Defaults follow the reference (-n 100, -t 0.001, -s 0.0935;
ArgumentsParser.cpp:6-10). At exit it prints the step count and the mean time
per step, as the reference's RenderTimer prints its average frame time
(src/RenderTimer/RenderTimer.cpp:77-94).
"""
from __future__ import annotations

import argparse
import sys
import time

import numpy as np

from . import NBodyError, ParticleSolverCUDA, ParticleSystem
from . import initializers as I
from . import io

VERSIONS = {8: "pp", 9: "bh"}


def parse(argv):
    ap = argparse.ArgumentParser(prog="python -m nbody_gb300", allow_abbrev=False)
    ap.add_argument("-v", "-version", dest="version", type=int, default=9)
    ap.add_argument("-n", dest="n", type=int, default=100)
    ap.add_argument("-i", "-init", dest="init", default="2")  # the reference defaults to the galaxy
    ap.add_argument("-t", "-time-step", dest="dt", type=float, default=0.001)
    ap.add_argument("-s", "-softening", dest="eps2", type=float, default=0.0935)
    ap.add_argument("-f", "-file", dest="file", default=None)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--theta", type=float, default=0.5, help="opening angle (the reference uses 0.5)")
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--integrator", choices=["cpu", "gpu_euler"], default="cpu")
    ap.add_argument("--keys", choices=["octree", "morton"], default="octree")
    ap.add_argument("--diagnostics-every", type=int, default=0)
    ap.add_argument("--save", default=None, help="write the final state (binary, lossless)")
    ap.add_argument("--dump", default=None, help="write the final state (the reference's text format)")
    return ap.parse_args(argv)


# -i values generated on the device by nbody_init_device.
DEVICE_INITS = {"1": "cube", "2": "galaxy", "4": "sphere", "5": "ball", "6": "cube_surface",
                "plummer": "plummer", "discs": "two_discs"}


def initial_system(args):
    """(host system or None, n, device initialiser kind or None)."""
    if args.file:
        with open(args.file, "rb") as f:
            head = f.read(8)
        system = io.load_binary(args.file) if head == io.MAGIC else io.read_text(args.file)
        return system, system.n, None
    init = str(args.init)
    if init == "3":
        p, v, m = I.lagrange()
        return ParticleSystem(p, v, m), 3, None
    if init in DEVICE_INITS:
        kind = DEVICE_INITS[init]
        n = args.n + (args.n % 2) if kind == "two_discs" else args.n
        return None, n, kind
    sys.stderr.write("Invalid initialization type\n")
    sys.exit(1)


def main(argv=None) -> int:
    args = parse(sys.argv[1:] if argv is None else argv)
    if args.version not in VERSIONS:
        sys.stderr.write("Invalid version\n")
        return 1
    if args.n <= 0:
        sys.stderr.write("Invalid number of particles\n")
        return 1
    system, n, device_kind = initial_system(args)
    try:
        solver = ParticleSolverCUDA(args.dt, args.eps2, n, mode=VERSIONS[args.version],
                                    theta2=args.theta * args.theta, device=args.device)
        solver.set_integrator(args.integrator)
        if VERSIONS[args.version] == "bh":
            solver.set_key_mode(args.keys)
        if device_kind is None:
            solver.upload(system)
        else:
            solver.init_device(device_kind, seed=args.seed)
            z = np.zeros((n, 4), np.float32)
            system = ParticleSystem(z, z.copy(), np.zeros(n, np.float32))
        print(f"version {args.version} ({VERSIONS[args.version]}), {n} bodies, dt {args.dt}, "
              f"eps2 {args.eps2}, {args.steps} steps", flush=True)
        t0 = time.perf_counter()
        done = 0
        every = args.diagnostics_every
        while done < args.steps:
            k = min(every, args.steps - done) if every > 0 else args.steps - done
            solver.step(k)
            done += k
            if every > 0:
                d = solver.diagnostics()
                print(f"step {done}: E {d['energy']:.9g} (K {d['kinetic']:.6g}, U {d['potential']:.6g}) "
                      f"P {np.linalg.norm(d['momentum']):.3g} L {np.linalg.norm(d['angular_momentum']):.6g}",
                      flush=True)
        solver.sync()
        secs = time.perf_counter() - t0
        solver.download(system, masses=device_kind is not None)
    except NBodyError as e:
        sys.stderr.write(f"{e}\n")
        return 1
    print(f"{done} steps, {1e3 * secs / max(done, 1):.4f} ms per step, "
          f"{system.n * done / max(secs, 1e-12):.4g} body-steps/s", flush=True)
    if args.save:
        io.save_binary(system, args.save)
    if args.dump:
        io.write_text(system, args.dump)
    return 0


if __name__ == "__main__":
    sys.exit(main())
