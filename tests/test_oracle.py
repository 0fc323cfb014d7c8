"""The CPU oracle checked against the reference's own outputs (golden fixtures
made by tests/golden/make_golden.py from the reference sources) and against
known answers. No GPU needed."""
import platform

import numpy as np
import pytest

from conftest import golden, rel_err_stats

X86 = platform.machine() in ("x86_64", "AMD64")
PP_FIXTURES = ["pp_ball_1024.npz", "pp_ball_1000.npz", "pp_small_1.npz", "pp_small_2.npz", "pp_small_3.npz",
               "pp_small_5.npz", "pp_small_127.npz", "pp_eps0_64.npz"]
BH_FIXTURES = ["bh_ball_2048.npz", "bh_ball_2048_theta06.npz", "bh_plummer_4096.npz"]


@pytest.mark.parametrize("name", PP_FIXTURES)
def test_port_pp_matches_reference(oracle, name):
    g = golden(name)
    dt, eps2 = float(g["dt"]), float(g["eps2"])
    p1, v1, a1, f1, _ = oracle.pp_run(g["pos"], g["vel"], g["acc"], g["mass"], dt, eps2, 1)
    pk, vk, ak, fk, _ = oracle.pp_run(g["pos"], g["vel"], g["acc"], g["mass"], dt, eps2, int(g["steps"]))
    if X86:
        # Same arithmetic, same compiler flags: bit-for-bit.
        for a, b in ((f1, g["force1"]), (p1, g["pos1"]), (v1, g["vel1"]), (a1, g["acc1"]), (pk, g["posk"]),
                     (vk, g["velk"]), (fk, g["forcek"])):
            np.testing.assert_array_equal(a, b)
    else:
        assert rel_err_stats(f1, g["force1"])[0] < 1e-6
        np.testing.assert_allclose(pk, g["posk"], rtol=1e-5, atol=1e-4)


def test_port_lagrange_matches_reference(oracle):
    g = golden("lagrange.npz")
    pk, vk, ak, fk, _ = oracle.pp_run(g["pos"], g["vel"], g["acc"], g["mass"], float(g["dt"]), float(g["eps2"]),
                                      int(g["steps"]))
    np.testing.assert_allclose(pk, g["posk"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(vk, g["velk"], rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("name", BH_FIXTURES)
def test_port_bh_matches_reference(oracle, name):
    g = golden(name)
    dt, eps2, th = float(g["dt"]), float(g["eps2"]), float(g["theta2"])
    p1, v1, a1, f1, info = oracle.bh_run(g["pos"], g["vel"], g["acc"], g["mass"], dt, eps2, 1, theta2=th, threads=1)
    assert info["rc"] == 0
    assert info["root_mass"] == pytest.approx(float(g["root_mass1"]), rel=1e-6)
    # Same tree (bit-identical topology and boxes with one thread); centres of
    # mass differ by a few ulps (the reference's compiler reorders the child
    # sums), so forces agree to ~1e-6.
    rms, mx = rel_err_stats(f1, g["force1"])
    assert rms < 2e-6 and mx < 5e-5, (rms, mx)
    pk, vk, ak, fk, info = oracle.bh_run(g["pos"], g["vel"], g["acc"], g["mass"], dt, eps2, int(g["steps"]),
                                         theta2=th, threads=1)
    scale = np.abs(g["posk"][:, :3]).max()
    assert np.abs(pk[:, :3] - g["posk"][:, :3]).max() < 1e-6 * scale
    rms, mx = rel_err_stats(fk, g["forcek"])
    assert rms < 2e-6 and mx < 5e-5, (rms, mx)


def test_port_bh_patched_equals_unpatched(oracle):
    g = golden("bh_ball_2048.npz")
    args = (g["pos"], g["vel"], g["acc"], g["mass"], float(g["dt"]), float(g["eps2"]), 2)
    a = oracle.bh_run(*args, threads=2, patched=False)
    b = oracle.bh_run(*args, threads=2, patched=True)
    np.testing.assert_array_equal(a[3], b[3])
    np.testing.assert_array_equal(a[0], b[0])


def test_port_bh_reports_reference_overflow(oracle):
    # A centrally concentrated input overflows -v 6's fixed per-task node
    # regions (src/Octree/ParallelOctreeCPU.cpp:27,38); the reference writes
    # past them, the port reports it, and the patched layout runs.
    from nbody_gb300 import initializers as I

    pos, vel, mass = I.plummer(4096, a=100.0, seed=12)
    r = oracle.bh_run(pos, vel, np.zeros_like(pos), mass, 0.0035, 40.0, 1, threads=2, patched=False)
    assert r[4]["rc"] == 4
    r = oracle.bh_run(pos, vel, np.zeros_like(pos), mass, 0.0035, 40.0, 1, threads=2, patched=True)
    assert r[4]["rc"] == 0
    assert r[4]["root_mass"] == pytest.approx(4096.0, rel=1e-6)


def test_direct_f64_two_body(oracle):
    pos = np.array([[0, 0, 0, 0], [3, 4, 0, 0]], np.float32)
    m = np.array([2.0, 5.0], np.float32)
    a = oracle.direct_f64(pos, m, 0.0)
    np.testing.assert_allclose(a[0], 5.0 * np.array([3, 4, 0]) / 125.0, rtol=1e-12)
    np.testing.assert_allclose(a[1], -2.0 * np.array([3, 4, 0]) / 125.0, rtol=1e-12)


def test_reference_pp_error_vs_f64(oracle):
    g = golden("pp_ball_1024.npz")
    a64 = oracle.direct_f64(g["pos"], g["mass"], float(g["eps2"]))
    rms, mx = rel_err_stats(g["force1"], a64)
    assert rms < 1e-5


# ------------------------------------------------------------ Morton / sort
def _glsl_expand_bits(v):
    """morton.glsl:37-43 (10-bit -> 30-bit spread), restated in Python."""
    v = (v * 0x00010001) & 0xFF0000FF
    v = (v * 0x00000101) & 0x0F00F00F
    v = (v * 0x00000011) & 0xC30C30C3
    v = (v * 0x00000005) & 0x49249249
    return v


def test_morton_matches_glsl_convention_on_10_bits(oracle):
    """On inputs with 10 significant bits per axis the 63-bit key is the
    reference's 30-bit key (morton.glsl:63: ex * 4 + ey * 2 + ez)."""
    rng = np.random.default_rng(0)
    bmin = np.zeros(3, np.float32)
    bmax = np.full(3, 1.0, np.float32)
    q = rng.integers(0, 1024, size=(500, 3))
    # grid points exactly representable: p = q / 1024 lands in cell q * 2^11 at 21 bits
    pos = np.zeros((500, 4), np.float32)
    pos[:, :3] = q / 1024.0
    keys = oracle.morton63(pos, bmin, bmax)
    for (qx, qy, qz), k in zip(q, keys):
        k30 = _glsl_expand_bits(int(qx)) * 4 + _glsl_expand_bits(int(qy)) * 2 + _glsl_expand_bits(int(qz))
        assert int(k) >> 33 == k30


def test_morton_corners_and_monotone(oracle):
    pos = np.array([[-1, -2, -3, 0], [1, 2, 3, 0], [0, 0, 0, 0], [1, -2, -3, 0]], np.float32)
    mn, mx = oracle.bbox(pos)
    keys = oracle.morton63(pos, mn, mx)
    assert keys[0] == 0
    assert keys[1] == (1 << 63) - 1
    assert keys[3] == int("100" * 21, 2)  # x high in every triple
    rng = np.random.default_rng(1)
    p = rng.uniform(-5, 5, size=(2000, 4)).astype(np.float32)
    p[:, 3] = 0
    mn, mx = oracle.bbox(p)
    k = oracle.morton63(p, mn, mx)
    # moving +x never lowers the key
    p2 = p.copy()
    p2[:, 0] = np.minimum(p[:, 0] + 0.5, mx[0])
    kx = np.array([int(v) >> 2 & 0x1249249249249249 for v in k], dtype=np.uint64)
    kx2 = np.array([int(v) >> 2 & 0x1249249249249249 for v in oracle.morton63(p2, mn, mx)], dtype=np.uint64)
    assert np.all(kx2 >= kx)


def test_octree_keys_follow_reference_descent(oracle):
    """Octree-descent keys vs a direct Python restatement of
    Octree::getNextNode / Octree::subdivide in float32, and they agree with the
    morton.glsl quantisation except within rounding of cell boundaries."""
    rng = np.random.default_rng(3)
    p = rng.uniform(-50, 70, size=(3000, 4)).astype(np.float32)
    p[:, 3] = 0
    mn, mx = oracle.bbox(p)
    keys = oracle.octree_keys(p, mn, mx)
    f = np.float32
    for i in range(0, 3000, 97):
        lo, hi, key = mn.copy(), mx.copy(), 0
        for _ in range(21):
            d = 0
            for a in range(3):
                c = f(lo[a] + f(f(hi[a] - lo[a]) / f(2)))
                up = not (p[i, a] < c)
                if up:
                    lo[a] = c
                else:
                    hi[a] = c
                d |= int(up) << (2 - a)
            key = (key << 3) | d
        assert int(keys[i]) == key
    mk = oracle.morton63(p, mn, mx)
    assert np.mean(keys >> np.uint64(33) == mk >> np.uint64(33)) > 0.99


def test_bbox_reference_seed_quirk(oracle):
    # max seeds are FLT_MIN (ParallelOctreeCPU.cpp:80): an all-negative axis keeps max = FLT_MIN
    pos = np.array([[-1, 1, -5, 0], [-2, 3, -4, 0]], np.float32)
    mn, mx = oracle.bbox(pos)
    assert mn.tolist() == [-2, 1, -5]
    assert mx[1] == 3
    assert mx[0] == np.finfo(np.float32).tiny and mx[2] == np.finfo(np.float32).tiny


def test_sort_stable(oracle):
    rng = np.random.default_rng(2)
    keys = rng.integers(0, 50, size=10000).astype(np.uint64) << np.uint64(40)
    ks, perm = oracle.sort_stable(keys)
    ref = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(perm, ref)
    np.testing.assert_array_equal(ks, keys[ref])
    big = rng.integers(0, 2**63, size=5000, dtype=np.uint64)
    ks, perm = oracle.sort_stable(big)
    np.testing.assert_array_equal(perm, np.argsort(big, kind="stable"))
