"""A C++ caller steps systems on the GPU through the C ABI.

The program below is compiled with g++ against include/nbody_gb300.h only
(no reference headers, no torch), linked with libnbody_gb300.so, and keeps
its bodies as the reference's ParticleSystem does: five host arrays of vec4
(positions, accelerations, velocities, masses, forces;
include/ParticleSystem.h:82-86 of the reference), the mass in the first
component. It runs the reference's golden cases through nbody_update_host,
one call per step as ParticleSimulation drives a solver, and the results are
compared with the reference's own outputs under the same bounds as the
Python-side golden tests (tests/test_pp_gpu.py, tests/test_bh_gpu.py).
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, rel_err_stats

pytestmark = pytest.mark.gpu

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "nbody_gb300.h"

struct vec4 { float x, y, z, w; };

// The reference's ParticleSystem arrays, host side.
struct Bodies {
    std::vector<vec4> positions, accelerations, velocities, masses, forces;
    explicit Bodies(size_t n) : positions(n), accelerations(n), velocities(n), masses(n), forces(n) {}
};

static bool read_all(const char *path, void *dst, size_t bytes) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    const bool ok = std::fread(dst, 1, bytes, f) == bytes;
    std::fclose(f);
    return ok;
}

static bool write_all(const char *path, const void *src, size_t bytes) {
    FILE *f = std::fopen(path, "wb");
    if (!f) return false;
    const bool ok = std::fwrite(src, 1, bytes, f) == bytes;
    std::fclose(f);
    return ok;
}

// usage: caller <mode 0|1> <n> <dt> <eps2> <theta2> <steps> <in.bin> <out.bin>
// in.bin: positions, velocities, accelerations, masses (n vec4 each);
// out.bin: positions, velocities, accelerations, forces after `steps` calls.
int main(int argc, char **argv) {
    if (argc != 9) return 2;
    const int mode = std::atoi(argv[1]);
    const long n = std::atol(argv[2]);
    const float dt = std::strtof(argv[3], nullptr), eps2 = std::strtof(argv[4], nullptr),
                theta2 = std::strtof(argv[5], nullptr);
    const int steps = std::atoi(argv[6]);
    Bodies b(static_cast<size_t>(n));
    const size_t bytes = static_cast<size_t>(n) * sizeof(vec4);
    std::vector<vec4> in(4 * static_cast<size_t>(n));
    if (!read_all(argv[7], in.data(), 4 * bytes)) return 3;
    for (long i = 0; i < n; ++i) {
        b.positions[i] = in[i];
        b.velocities[i] = in[n + i];
        b.accelerations[i] = in[2 * n + i];
        b.masses[i] = in[3 * n + i];
    }
    nbody_ctx *ctx = nullptr;
    int rc = nbody_create(&ctx, 0, mode, n, dt, eps2, theta2);
    if (rc != NBODY_OK) {
        std::printf("create: %s\n", nbody_status_string(rc));
        return 4;
    }
    for (int s = 0; s < steps && rc == NBODY_OK; ++s)
        rc = nbody_update_host(ctx, &b.positions[0].x, &b.velocities[0].x, &b.accelerations[0].x,
                               &b.masses[0].x, &b.forces[0].x, 1);
    if (rc != NBODY_OK) {
        std::printf("update: %s %s\n", nbody_status_string(rc), nbody_last_error(ctx));
        nbody_destroy(ctx);
        return 5;
    }
    std::printf("eps2 %g\n", nbody_get_squared_softening(ctx));
    nbody_destroy(ctx);
    std::vector<vec4> out(4 * static_cast<size_t>(n));
    for (long i = 0; i < n; ++i) {
        out[i] = b.positions[i];
        out[n + i] = b.velocities[i];
        out[2 * n + i] = b.accelerations[i];
        out[3 * n + i] = b.forces[i];
    }
    return write_all(argv[8], out.data(), 4 * bytes) ? 0 : 6;
}
"""


@pytest.fixture(scope="module")
def caller(nb, tmp_path_factory):
    d = tmp_path_factory.mktemp("cpp_caller")
    src = d / "caller.cpp"
    src.write_text(PROGRAM)
    exe = d / "caller"
    libdir = os.path.dirname(nb.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", f"-I{ROOT}/include", str(src), f"-L{libdir}", "-lnbody_gb300",
           f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run(exe, tmp_path, mode, g, steps):
    n = len(g["mass"])
    masses = np.zeros((n, 4), np.float32)
    masses[:, 0] = g["mass"]
    inp = tmp_path / "in.bin"
    out = tmp_path / "out.bin"
    np.concatenate([g["pos"], g["vel"], g["acc"], masses]).astype(np.float32).tofile(inp)
    theta2 = float(g["theta2"]) if "theta2" in g else 0.25
    args = [str(exe), str(mode), str(n), repr(float(g["dt"])), repr(float(g["eps2"])), repr(theta2), str(steps),
            str(inp), str(out)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith(f"eps2 {float(g['eps2']):g}"), r.stdout
    res = np.fromfile(out, np.float32).reshape(4, n, 4)
    return res[0], res[1], res[2], res[3]


def test_cpp_caller_direct_sum_matches_reference_golden(nb, cuda, caller, tmp_path):
    g = golden("pp_ball_1024.npz")
    pos, vel, acc, force = _run(caller, tmp_path, nb.MODE_PP, g, int(g["steps"]))
    rms, mx = rel_err_stats(force, g["forcek"])
    assert rms <= 1e-5 and mx <= 1e-3, (rms, mx)
    np.testing.assert_allclose(pos, g["posk"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(vel, g["velk"], rtol=1e-5, atol=1e-5)
    np.testing.assert_array_equal(acc, force)
    assert np.all(pos[:, 3] == 0)


def test_cpp_caller_barnes_hut_matches_reference_golden(nb, cuda, caller, tmp_path):
    g = golden("bh_ball_2048.npz")
    pos, vel, acc, force = _run(caller, tmp_path, nb.MODE_BH, g, int(g["steps"]))
    scale = np.abs(g["posk"][:, :3]).max()
    assert np.abs(pos[:, :3] - g["posk"][:, :3]).max() <= 1e-6 * scale
    rms, mx = rel_err_stats(force, g["forcek"])
    assert rms <= 2e-6 and mx <= 1e-3, (rms, mx)
    np.testing.assert_allclose(vel, g["velk"], rtol=1e-4, atol=1e-5)
    assert np.all(pos[:, 3] == 0)
