"""The C++ drop-in (include/ParticleSolverCUDA.h) compiles against the
reference's own headers (ParticleSolver.h, ParticleSystem.h; glm and GL
satisfied by the headless shim) and links with the reference's
ParticleSystem objects and libnbody_gb300.so. Where a GPU is present the
program also steps a system and prints its forces. Needs the reference
checkout (it is not on the GPU host), so it skips there."""
import os
import subprocess

import pytest

import pyoracle
from conftest import ROOT

REF = pyoracle.reference_dir()

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "ParticleSolverCUDA.h"

int main() {
    std::vector<Particle> ps;
    for (int i = 0; i < 64; ++i)
        ps.emplace_back(glm::vec3(float(i % 4), float((i / 4) % 4), float(i / 16)), glm::vec3(0.f), 1.0f + i);
    ParticleSystem sys(ps, false);
    ParticleSolver *solver = nullptr;
    try {
        solver = new ParticleSolverCUDA(0.01f, 0.5f, 64, ParticleSolverCUDA::Mode::DirectSum);
    } catch (const std::runtime_error &e) {
        std::printf("no-device %s\n", e.what());
        return 0;
    }
    solver->updateParticlePositions(&sys);
    std::printf("uses_gpu %d eps2 %g f0 %g %g %g\n", int(solver->usesGPU()), solver->getSquaredSoftening(),
                sys.getForces()[0].x, sys.getForces()[0].y, sys.getForces()[0].z);
    delete solver;
    return 0;
}
"""


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "include")), reason="reference checkout absent")
def test_adapter_compiles_links_and_runs(nb, oracle, tmp_path):
    oracle.build(reference=True)
    objdir = os.path.join(ROOT, "oracle", "_ref", "obj")
    objs = [os.path.join(objdir, "src", "ParticleSystem", "ParticleSystem.o"),
            os.path.join(objdir, "src", "Particle", "Particle.o"),
            os.path.join(objdir, "src", "OpenGLBuffer", "OpenGLBuffer.o"),
            os.path.join(objdir, "gl_stub.o")]
    src = tmp_path / "adapter.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "adapter"
    libdir = os.path.dirname(nb.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", f"-I{REF}/include", f"-I{ROOT}/oracle/shim", f"-I{ROOT}/include",
           str(src), *objs, f"-L{libdir}", "-lnbody_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    try:
        import torch

        gpu = torch.cuda.is_available()
    except ImportError:
        gpu = False
    if gpu:
        assert out.stdout.startswith("uses_gpu 0"), out.stdout
    else:
        assert out.stdout.startswith("no-device") or out.stdout.startswith("uses_gpu 0"), out.stdout
