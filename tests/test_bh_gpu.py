"""Barnes-Hut CUDA path vs the oracle.

Bit-exact: the root box and the 63-bit Morton keys (vs the C restatement of
morton.glsl), and the sort permutation (vs numpy's stable argsort). Structure:
root mass, pre-order links, each body in exactly one leaf, cell sides equal to
the reference's FP32 box halving. Accelerations vs the reference's own -v 6
outputs (golden fixtures) and vs the port at larger n, with the tolerances
stated per test; FP64 direct-sum error reported against the reference's.
"""
import numpy as np
import pytest

from conftest import golden, rel_err_stats

pytestmark = pytest.mark.gpu

BH_FIXTURES = ["bh_ball_2048.npz", "bh_ball_2048_theta06.npz", "bh_plummer_4096.npz"]


def check_large(f, ref, rms_tol=3e-5, p999_tol=5e-4, max_tol=2e-3):
    """Parity bound at large n. Cells, sides and the opening test are the
    reference's, but centres of mass are summed in another order (pairwise
    over the radix tree instead of the reference's per-cell sum over up to 8
    children), so a few opening decisions land on the other side of
    s^2 < theta^2 d^2 and move that body's force by about the Barnes-Hut
    error of one cell (~1e-4 .. 1e-3), mostly in the dense core. Bound: RMS
    <= rms_tol, 99.9th percentile <= p999_tol, worst body <= max_tol."""
    got = np.asarray(f, np.float64)[:, :3]
    r = np.asarray(ref, np.float64)[:, :3]
    e = np.linalg.norm(got - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-30)
    rms = float(np.sqrt(np.mean(e * e)))
    p999 = float(np.percentile(e, 99.9))
    print(f"parity: rms={rms:.3e} p99.9={p999:.3e} max={e.max():.3e} frac>1e-5={(e > 1e-5).mean():.2e}")
    assert rms <= rms_tol and p999 <= p999_tol and e.max() <= max_tol, (rms, p999, e.max())


def solver_for(nb, n, eps2=40.0, theta2=0.25, dt=0.0035):
    return nb.ParticleSolverCUDA(dt, eps2, n, mode="bh", theta2=theta2)


def bh_forces(nb, torch, pos, mass, eps2=40.0, theta2=0.25):
    from nbody_gb300 import initializers as I

    n = len(mass)
    s = solver_for(nb, n, eps2, theta2)
    pm = torch.from_numpy(I.pos_mass(pos, mass)).cuda()
    f = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    s.bh_forces_device(pm, f)
    s.sync()
    return f.cpu().numpy(), s


# ------------------------------------------------------------------ keys / box
@pytest.mark.parametrize("mode", ["octree", "morton"])
@pytest.mark.parametrize("kind", ["ball", "plummer", "negative_axis", "flat"])
def test_box_and_keys_bit_exact(nb, cuda, oracle, kind, mode):
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 200_003
    if kind == "ball":
        pos, _, mass = I.uniform_ball(n, seed=21)
    elif kind == "plummer":
        pos, _, mass = I.plummer(n, seed=22)
    elif kind == "negative_axis":  # all x < 0: the reference's max seed FLT_MIN stays
        pos, _, mass = I.uniform_ball(n, seed=23)
        pos[:, 0] = -np.abs(pos[:, 0]) - 1.0
    else:  # zero extent in z
        pos, _, mass = I.uniform_ball(n, seed=24)
        pos[:, 2] = 3.0
    s = solver_for(nb, n)
    s.set_key_mode(mode)
    pm = torch.from_numpy(I.pos_mass(pos, mass)).cuda()
    keys = torch.zeros(n, dtype=torch.int64, device="cuda")
    box = torch.zeros(6, dtype=torch.float32, device="cuda")
    s.bh_keys_device(pm, keys, box)
    s.sync()
    mn, mx = oracle.bbox(pos)
    np.testing.assert_array_equal(box.cpu().numpy(), np.concatenate([mn, mx]))
    ref = oracle.octree_keys(pos, mn, mx) if mode == "octree" else oracle.morton63(pos, mn, mx)
    np.testing.assert_array_equal(keys.cpu().numpy().view(np.uint64), ref)


# ------------------------------------------------------------------------ sort
@pytest.mark.parametrize("n", [1, 2, 3, 4095, 4096, 4097, 100_000, 1 << 20])
def test_sort_is_stable_and_exact(nb, cuda, n):
    torch = cuda
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << 63, size=n, dtype=np.uint64)
    keys[rng.random(n) < 0.3] = np.uint64(12345)  # many duplicates
    keys[: n // 7] &= np.uint64(0xFFFF)           # many shared high digits
    vals = np.arange(n, dtype=np.uint32)
    s = solver_for(nb, max(n, 2))
    kt = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    vt = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    s.sort_pairs_device(kt, vt, n)
    s.sync()
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(kt.cpu().numpy().view(np.uint64), keys[order])
    np.testing.assert_array_equal(vt.cpu().numpy().view(np.uint32), order.astype(np.uint32))


def test_sort_permutation_of_morton_keys_matches_oracle(nb, cuda, oracle):
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 1 << 20
    pos, _, mass = I.plummer(n, seed=31)
    mn, mx = oracle.bbox(pos)
    keys = oracle.morton63(pos, mn, mx)
    ks, perm = oracle.sort_stable(keys)
    s = solver_for(nb, n)
    kt = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    vt = torch.arange(n, dtype=torch.int32, device="cuda")
    s.sort_pairs_device(kt, vt, n)
    s.sync()
    np.testing.assert_array_equal(vt.cpu().numpy().view(np.uint32), perm)
    np.testing.assert_array_equal(kt.cpu().numpy().view(np.uint64), ks)


# ------------------------------------------------------------------------ tree
def reference_cell_side2(key, level, box):
    """Octree::subdivide box halving (src/Octree/Octree.cpp:159-231) in float32."""
    mn = np.array(box[:3], np.float32)
    mx = np.array(box[3:], np.float32)
    half = np.float32(0.5)
    for lv in range(1, level + 1):
        d = (int(key) >> (63 - 3 * lv)) & 7
        for a in range(3):
            w = np.float32(mx[a] - mn[a])
            c = np.float32(mn[a] + np.float32(w * half))
            if (d >> (2 - a)) & 1:
                mn[a] = c
            else:
                mx[a] = c
    sd = (mx - mn).astype(np.float32)
    sv = np.float32(max(max(sd[0], sd[1]), sd[2]))
    return np.float32(sv * sv)


@pytest.mark.parametrize("kind", ["ball", "plummer", "duplicates"])
def test_tree_invariants(nb, cuda, oracle, kind):
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 50_000
    if kind == "plummer":
        pos, _, mass = I.plummer(n, seed=41)
    else:
        pos, _, mass = I.uniform_ball(n, seed=42)
        if kind == "duplicates":
            pos[1000:1100] = pos[1000]           # a bucket of 100 identical positions
            pos[5:8] = pos[4]
    _, s = bh_forces(nb, torch, pos, mass)
    cm, meta, box = s.bh_tree()
    m = len(cm)
    assert n <= m <= 2 * n
    # root mass
    assert cm[0, 3] == pytest.approx(float(mass.astype(np.float64).sum()), rel=1e-5)
    s2 = meta[:, 0].view(np.float32)
    nxt, first, cnt = meta[:, 1], meta[:, 2], meta[:, 3]
    idx = np.arange(m)
    assert np.all(nxt > idx) and nxt[0] == m
    leaf = s2 < 0
    cell = ~leaf
    # a cell's first child is the next record and lies inside it
    assert np.all(nxt[idx[cell] + 1] <= nxt[cell])
    # bodies: every sorted body in exactly one leaf, leaves in body order
    covered = np.zeros(n, np.int64)
    for f, c in zip(first[leaf], cnt[leaf]):
        covered[f:f + c] += 1
    assert np.all(covered == 1)
    assert np.all(np.diff(first[leaf]) > 0)
    # a cell flagged terminal (meta.w < 0) has only leaves below it, -meta.w of them
    term = cell & (cnt < 0)
    assert term.sum() > 0
    for i in np.flatnonzero(term)[:2000]:
        sub = np.arange(i + 1, nxt[i])
        assert np.all(leaf[sub]), i
        assert -cnt[i] == cnt[sub].sum()
    assert np.all(cnt[cell & ~term] == 0)
    # cell masses equal the sum of the leaves in their subtree
    leaf_mass = np.where(leaf, cm[:, 3].astype(np.float64), 0.0)
    csum = np.concatenate([[0.0], np.cumsum(leaf_mass)])
    sub = csum[nxt[cell]] - csum[idx[cell]]
    np.testing.assert_allclose(cm[cell, 3], sub, rtol=1e-5)
    # cell sides: the reference's FP32 halving of the root box
    mn, mx = oracle.bbox(pos)
    np.testing.assert_array_equal(box, np.concatenate([mn, mx]))
    keys = np.sort(oracle.octree_keys(pos, mn, mx))
    rng = np.random.default_rng(0)
    for i in rng.choice(np.flatnonzero(cell), size=min(300, int(cell.sum())), replace=False):
        body = first[i]
        # level of the cell: deepest level whose prefix all its bodies share
        lo, hi = first[i], None
        j = i + 1
        last_leaf = np.flatnonzero(leaf[i:nxt[i]])[-1] + i
        hi = first[last_leaf] + cnt[last_leaf] - 1
        x = int(keys[lo]) ^ int(keys[hi])
        prefix = 63 - x.bit_length()
        level = min(21, prefix // 3)
        assert s2[i] == reference_cell_side2(keys[body], level, box), (i, level)


@pytest.mark.parametrize("kind", ["plummer", "duplicates"])
def test_upsweep_schedules_agree(nb, cuda, monkeypatch, kind):
    """The climbing upsweep (one launch, atomic arrivals) and the level schedule
    (one launch per octree level) build the same records bit for bit, buckets
    of identical positions included, and so the same forces and steps."""
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 50_000
    if kind == "plummer":
        pos, vel, mass = I.plummer(n, seed=43)
    else:
        pos, vel, mass = I.uniform_ball(n, seed=44)
        pos[2000:2100] = pos[2000]
        pos[7:9] = pos[6]
    out = {}
    for sched in ("climb", "levels"):
        monkeypatch.setenv("NBODY_UPSWEEP", sched)
        f, s = bh_forces(nb, torch, pos, mass)
        out[sched] = (f, *s.bh_tree())
        s.close()
        sysm = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
        s = solver_for(nb, n)
        s.update_particle_positions(sysm, steps=2)
        s.close()
        out[sched + " steps"] = (sysm.positions, sysm.velocities, sysm.accelerations)
    for a, b in zip(out["climb"], out["levels"]):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(out["climb steps"], out["levels steps"]):
        np.testing.assert_array_equal(a, b)


# ---------------------------------------------------------------------- forces
@pytest.mark.parametrize("name", BH_FIXTURES)
def test_bh_forces_match_reference_golden(nb, cuda, oracle, name):
    """The reference's -v 6 accelerations (one thread, same inputs). The cells,
    their sides and the opening test are the reference's; what differs is the
    hardware rsqrt instead of pow/divide, the summation order of centres of
    mass, and the reference's merging of bodies closer than sqrt(1e-3). Bound:
    per-body relative error RMS <= 2e-6 and max <= 1e-3."""
    torch = cuda
    g = golden(name)
    f, _ = bh_forces(nb, torch, g["pos"], g["mass"], float(g["eps2"]), float(g["theta2"]))
    rms, mx = rel_err_stats(f, g["force1"])
    assert rms <= 2e-6 and mx <= 1e-3, (rms, mx)
    # and against the port
    pf = oracle.bh_run(g["pos"], g["vel"], g["acc"], g["mass"], float(g["dt"]), float(g["eps2"]), 1,
                       theta2=float(g["theta2"]), threads=0)[3]
    rms, mx = rel_err_stats(f, pf)
    assert rms <= 2e-6 and mx <= 1e-3, (rms, mx)


@pytest.mark.parametrize("name", BH_FIXTURES)
def test_bh_steps_match_reference_golden(nb, cuda, name):
    g = golden(name)
    n = len(g["mass"])
    sysm = nb.ParticleSystem(g["pos"].copy(), g["vel"].copy(), g["mass"], g["acc"].copy())
    s = solver_for(nb, n, float(g["eps2"]), float(g["theta2"]), float(g["dt"]))
    s.update_particle_positions(sysm, steps=int(g["steps"]))
    scale = np.abs(g["posk"][:, :3]).max()
    assert np.abs(sysm.positions[:, :3] - g["posk"][:, :3]).max() <= 1e-6 * scale
    rms, mx = rel_err_stats(sysm.forces, g["forcek"])
    assert rms <= 2e-6 and mx <= 1e-3, (rms, mx)
    np.testing.assert_allclose(sysm.velocities, g["velk"], rtol=1e-4, atol=1e-5)
    assert np.all(sysm.positions[:, 3] == 0)


def test_bh_plummer_vs_port_and_fp64(nb, cuda, oracle):
    """262,144-body Plummer sphere (a = 100, truncated at 20a): against the port
    (patched capacities; the reference's fixed regions overflow here) with the
    large-n bound of check_large, and the FP64 direct sum on a sample: the
    GPU's FP64 error must match the port's to within 10%."""
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 1 << 18
    pos, vel, mass = I.plummer(n, seed=51)
    f, _ = bh_forces(nb, torch, pos, mass)
    pf = oracle.bh_run(pos, vel, np.zeros_like(pos), mass, 0.0035, 40.0, 1, theta2=0.25, patched=True)[3]
    check_large(f, pf)
    idx = np.random.default_rng(5).choice(n, 2048, replace=False)
    a64 = oracle.direct_f64(pos, mass, 40.0, idx=idx)
    e_gpu = rel_err_stats(f[idx], a64)[0]
    e_port = rel_err_stats(pf[idx], a64)[0]
    assert e_gpu <= 1.1 * e_port + 1e-6, (e_gpu, e_port)


def test_bh_theta_zero_is_direct_sum(nb, cuda, oracle):
    """theta -> 0 opens every cell: the tree walk reduces to the direct sum."""
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 3000
    pos, _, mass = I.uniform_ball(n, seed=52)
    f, _ = bh_forces(nb, torch, pos, mass, theta2=1e-12)
    rms, mx = rel_err_stats(f, oracle.pp_forces(pos, mass, 40.0))
    assert rms <= 1e-5 and mx <= 1e-3, (rms, mx)


@pytest.mark.parametrize("n", [1, 2, 3, 33, 4097])
def test_bh_small_sizes(nb, cuda, oracle, n):
    torch = cuda
    from nbody_gb300 import initializers as I

    pos, _, mass = I.uniform_ball(n, seed=53 + n)
    f, _ = bh_forces(nb, torch, pos, mass)
    if n == 1:
        assert np.all(f == 0)
        return
    pf = oracle.bh_run(pos, np.zeros_like(pos), np.zeros_like(pos), mass, 0.0035, 40.0, 1, theta2=0.25,
                       patched=True)[3]
    rms, mx = rel_err_stats(f, pf)
    assert rms <= 2e-6 and mx <= 1e-3, (rms, mx)


def test_bh_coincident_bodies(nb, cuda, oracle):
    """Bodies at identical positions share one leaf and interact one by one;
    pairs at zero distance are skipped (the reference's d^2 > 0 test)."""
    torch = cuda
    n = 64
    rng = np.random.default_rng(7)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-10, 10, size=(n, 3))
    pos[10:20] = pos[10]
    mass = rng.uniform(1, 2, n).astype(np.float32)
    f, _ = bh_forces(nb, torch, pos, mass, theta2=1e-12)
    ref = oracle.direct_f64(pos, mass, 40.0)  # the FP64 sum skips only j == i; coincident pairs add 0
    rms, mx = rel_err_stats(f, ref)
    assert rms <= 1e-5, (rms, mx)
    same = np.zeros((n, 4), np.float32)
    same[:, :3] = 5.0
    f, _ = bh_forces(nb, torch, same, mass)
    assert np.all(f == 0)


def test_bh_resident_steps_equal_host_calls_and_deterministic(nb, cuda):
    from nbody_gb300 import initializers as I

    n = 30_000
    pos, vel, mass = I.plummer(n, seed=61)
    a = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    s = solver_for(nb, n)
    for _ in range(3):
        s.update_particle_positions(a)
    b = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    s.upload(b)
    s.step(3)
    s.download(b)
    for x, y in ((a.positions, b.positions), (a.velocities, b.velocities), (a.forces, b.forces)):
        np.testing.assert_array_equal(x, y)


def test_bh_ten_steps_vs_port(nb, cuda, oracle):
    """Ten steps of a 65,536-body Plummer sphere against the port (check_large)."""
    from nbody_gb300 import initializers as I

    n = 1 << 16
    pos, vel, mass = I.plummer(n, seed=62)
    sysm = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    solver_for(nb, n).update_particle_positions(sysm, steps=10)
    pk, vk, ak, fk, info = oracle.bh_run(pos, vel, np.zeros_like(pos), mass, 0.0035, 40.0, 10, theta2=0.25,
                                         patched=True)
    assert info["rc"] == 0
    check_large(sysm.forces, fk)
    scale = np.abs(pk[:, :3]).max()
    assert np.abs(sysm.positions[:, :3] - pk[:, :3]).max() <= 1e-6 * scale


@pytest.mark.parametrize("kind,n,eps2,theta2", [("plummer", 1 << 17, 40.0, 0.25), ("uniform_ball", 100_000, 40.0, 0.36),
                                                ("plummer", 50_000, 0.0, 0.25)])
def test_walk_forms_accept_the_same_pairs(nb, cuda, monkeypatch, kind, n, eps2, theta2):
    """The cell walk (default) decides records for whole sets of bodies from
    their box; the union walk decides every record body by body. Both must give
    every body exactly the records its own reference walk accepts: the pair
    counts of one step are equal, and the forces differ only by summation
    order (eps^2 = 0 exercises the explicit zero-distance tests)."""
    out = {}
    for form in ("union", "cell"):
        monkeypatch.setenv("NBODY_BH_WALK", form)
        s = nb.ParticleSolverCUDA(0.0035, eps2, n, mode="bh", theta2=theta2)
        s.init_device(kind, seed=77)
        s.bh_counters(True)
        s.step(1)
        pairs, _ = s.bh_counters(False)
        z = np.zeros((n, 4), np.float32)
        sysm = nb.ParticleSystem(z.copy(), z.copy(), np.zeros(n, np.float32), z.copy())
        s.download(sysm)
        s.close()
        out[form] = (pairs, sysm.forces.copy())
    assert out["cell"][0] == out["union"][0] > 0
    rms, mx = rel_err_stats(out["cell"][1], out["union"][1])
    assert rms <= 1e-5 and mx <= 1e-3, (rms, mx)
