"""Headless run loop: python -m nbody_gb300 [-v version] [-n numParticles] [-i init]
[-t timeStep] [-s squaredSoftening] [-f filePath] [--steps K] ...

Mirrors the reference's command line (src/ArgumentsParser/ArgumentsParser.cpp:49-106,
long forms -version/-init/-time-step/-softening/-file) with the GPU solver
registered as two new versions, and replaces its window and render loop
(src/RenderLoop/RenderLoop.cpp:12-35) by a fixed number of steps:

  -v 8   direct sum on the GPU   (-v 2 semantics: ParticleSolverCPUParallel)
  -v 9   Barnes-Hut on the GPU   (-v 6 semantics: ParticleSolverBHutCPUParallel)

Versions 1-7 are the reference's own CPU and OpenGL solvers and are not part of
this program. Initialisers: -i 3 (the reference's Lagrange triangle), -i 5
(uniform ball), -f FILE (the reference's text format, or this library's
lossless binary format), and --init plummer / discs for the benchmark
workloads. Defaults follow the reference (-n 100, -t 0.001, -s 0.0935;
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
    ap.add_argument("-i", "-init", dest="init", default="5")
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


def initial_system(args) -> ParticleSystem:
    if args.file:
        with open(args.file, "rb") as f:
            head = f.read(8)
        return io.load_binary(args.file) if head == io.MAGIC else io.read_text(args.file)
    init = str(args.init)
    if init == "3":
        p, v, m = I.lagrange()
    elif init in ("5", "ball"):
        p, v, m = I.uniform_ball(args.n, seed=args.seed)
    elif init == "plummer":
        p, v, m = I.plummer(args.n, seed=args.seed)
    elif init == "discs":
        p, v, m = I.two_discs(max(1, (args.n - 2) // 2), seed=args.seed)
    else:
        sys.stderr.write("Invalid initialization type\n")
        sys.exit(1)
    return ParticleSystem(p, v, m)


def main(argv=None) -> int:
    args = parse(sys.argv[1:] if argv is None else argv)
    if args.version not in VERSIONS:
        sys.stderr.write("Invalid version\n")
        return 1
    if args.n <= 0:
        sys.stderr.write("Invalid number of particles\n")
        return 1
    system = initial_system(args)
    try:
        solver = ParticleSolverCUDA(args.dt, args.eps2, system.n, mode=VERSIONS[args.version],
                                    theta2=args.theta * args.theta, device=args.device)
        solver.set_integrator(args.integrator)
        if VERSIONS[args.version] == "bh":
            solver.set_key_mode(args.keys)
        solver.upload(system)
        print(f"version {args.version} ({VERSIONS[args.version]}), {system.n} bodies, dt {args.dt}, "
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
        solver.download(system)
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
