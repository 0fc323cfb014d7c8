"""Host-layout calls with page-locked host buffers.

nbody_upload / nbody_download read and write page-locked, mapped host buffers
in place with one kernel each (n-body_gb300/csrc/hostio.cu) instead of a
cudaMemcpyAsync per array; pageable buffers keep the copy path. Both paths
move the same values: every array must match bit for bit, for the direct sum
and for Barnes-Hut (whose resident state is in sorted order and is scattered
back through the body ids), and when only some buffers are page-locked; the
ensemble calls (nbody_ensemble_upload / _download) likewise. A buffer that is
page-locked over only part of its length takes the copy path.
"""
import ctypes
import mmap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pin(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()


def _system(nb, torch, pos, vel, mass, pinned):
    s = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
    if pinned == "all":
        for name in ("positions", "velocities", "accelerations", "masses", "forces"):
            setattr(s, name, _pin(torch, getattr(s, name)))
    elif pinned == "some":
        s.positions = _pin(torch, s.positions)
        s.forces = _pin(torch, s.forces)
    return s


def _same(a, b):
    for name in ("positions", "velocities", "accelerations", "forces"):
        np.testing.assert_array_equal(getattr(a, name), getattr(b, name), err_msg=name)


@pytest.mark.parametrize("mode,n,steps", [("pp", 5000, 3), ("pp", 1, 1), ("bh", 20000, 2), ("bh", 777, 3)])
def test_pinned_and_pageable_paths_agree(nb, cuda, mode, n, steps):
    torch = cuda
    from nbody_gb300 import initializers as I

    pos, vel, mass = I.plummer(n, a=50.0, seed=n) if n > 1 else I.uniform_ball(n, seed=1)
    out = {}
    for pinned in ("none", "all", "some"):
        s = _system(nb, torch, pos, vel, mass, pinned)
        solver = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode=mode, theta2=0.25)
        solver.update_particle_positions(s, steps=steps)
        solver.update_particle_positions(s)  # host state in, again
        solver.close()
        out[pinned] = s
    _same(out["all"], out["none"])
    _same(out["some"], out["none"])
    assert np.all(out["all"].positions[:, 3] == 0)


def test_resident_download_to_pinned_after_sorted_steps(nb, cuda):
    """Barnes-Hut state stays in sorted order between steps; a download into
    page-locked buffers must scatter it back to the caller's order."""
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 12345
    pos, vel, mass = I.plummer(n, a=100.0, seed=9)
    solver = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="bh", theta2=0.25)
    solver.upload(_system(nb, torch, pos, vel, mass, "all"))
    solver.step(4)
    a = _system(nb, torch, np.zeros_like(pos), np.zeros_like(vel), mass, "none")
    b = _system(nb, torch, np.zeros_like(pos), np.zeros_like(vel), mass, "all")
    solver.download(a)
    solver.download(b)
    solver.close()
    _same(a, b)


def test_upload_without_velocities_zeroes_them(nb, cuda):
    """nbody_upload with null velocity / acceleration buffers starts them at
    zero on both paths."""
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 3000
    pos, vel, mass = I.uniform_ball(n, seed=4)
    res = []
    for pinned in ("none", "all"):
        s = _system(nb, torch, pos, vel + 1.0, mass, pinned)
        solver = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="pp")
        p = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
        assert nb.lib().nbody_upload(solver._ctx, p(s.positions), None, None, p(s.masses)) == nb.OK
        solver.step(1)
        solver.download(s)
        solver.close()
        res.append(s)
    _same(res[0], res[1])
    ref = nb.ParticleSystem(pos.copy(), np.zeros_like(vel), mass)
    nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="pp").update_particle_positions(ref)
    np.testing.assert_array_equal(res[0].positions, ref.positions)


def test_ensemble_pinned_and_pageable_paths_agree(nb, cuda):
    """nbody_ensemble_upload / _download take the same in-place path for
    page-locked buffers: direct-sum and Barnes-Hut systems (the latter scattered
    back from key order), masses included, match the copy path bit for bit."""
    torch = cuda
    from nbody_gb300 import initializers as I

    sizes = [700, 5000, 1]
    res = {}
    for pinned in ("none", "all", "some"):
        with nb.Ensemble(crossover=2048) as ens:
            ids = []
            for k, n in enumerate(sizes):
                sid = ens.add(n, 0.0035, 40.0, 0.25)
                pos, vel, mass = I.plummer(n, a=50.0, seed=70 + k) if n > 1 else I.uniform_ball(n, seed=3)
                ens.upload(sid, _system(nb, torch, pos, vel, mass, pinned))
                ids.append((sid, n))
            ens.step(3)
            outs = []
            for sid, n in ids:
                z = np.zeros((n, 4), np.float32)
                o = _system(nb, torch, z[:, :3].copy(), z.copy(), np.zeros(n, np.float32), pinned)
                ens.download(sid, o)
                outs.append(o)
            res[pinned] = outs
    for a, b, c in zip(res["none"], res["all"], res["some"]):
        for name in ("positions", "velocities", "accelerations", "masses"):
            np.testing.assert_array_equal(getattr(a, name), getattr(b, name), err_msg=name)
            np.testing.assert_array_equal(getattr(a, name), getattr(c, name), err_msg=name)


def test_partly_page_locked_buffer_takes_the_copy_path(nb, cuda):
    """The in-place kernels touch all n float4 of a buffer through its mapped
    address, so they are used only when the page-locked range holds all of
    them. A buffer registered over its first half goes to cudaMemcpyAsync,
    which on this driver refuses a range that leaves the registered memory:
    the call then reports a CUDA error on the host (nothing is read past the
    registration on the device), and the solver stays usable."""
    torch = cuda
    from nbody_gb300 import initializers as I

    n = 4096
    nbytes = n * 16
    L = nb.lib()
    page = mmap.PAGESIZE
    buf = mmap.mmap(-1, nbytes + page)
    arr = np.frombuffer(buf, dtype=np.float32, count=n * 4).reshape(n, 4)
    ptr = arr.ctypes.data
    assert ptr % page == 0
    assert L.nbody_host_in_place(ctypes.c_void_p(ptr), nbytes, 0) == 0  # pageable
    half = nbytes // 2
    cudart = torch.cuda.cudart()
    err = cudart.cudaHostRegister(ptr, half, 0)
    assert int(err) == 0, err
    try:
        assert L.nbody_host_in_place(ctypes.c_void_p(ptr), half, 0) == 1
        assert L.nbody_host_in_place(ctypes.c_void_p(ptr), nbytes, 0) == 0
        assert L.nbody_host_in_place(ctypes.c_void_p(ptr + half - 16), 32, 0) == 0
        pinned = _pin(torch, np.zeros((n, 4), np.float32))
        assert L.nbody_host_in_place(ctypes.c_void_p(pinned.ctypes.data), nbytes, 0) == 1
        assert L.nbody_host_in_place(None, nbytes, 0) == nb.ERR_ARG

        pos, vel, mass = I.plummer(n, a=50.0, seed=31)
        ref = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
        solver = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="bh", theta2=0.25)
        solver.update_particle_positions(ref, steps=2)
        part = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
        arr[:] = part.positions
        part.positions = arr
        try:
            solver.update_particle_positions(part, steps=2)
        except nb.NBodyError as e:
            assert e.status == nb.ERR_CUDA, e
        else:
            _same(part, ref)
        solver.close()
        again = nb.ParticleSystem(pos.copy(), vel.copy(), mass)
        solver = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="bh", theta2=0.25)
        solver.update_particle_positions(again, steps=2)
        solver.close()
        _same(again, ref)
    finally:
        assert int(cudart.cudaHostUnregister(ptr)) == 0


@pytest.mark.parametrize("mode,n", [("bh", 30_000), ("pp", 5_000)])
@pytest.mark.parametrize("pinned", ["all", "none"])
def test_graph_replayed_steps_match_direct_launches(nb, cuda, monkeypatch, pinned, mode, n):
    """Steps replayed as CUDA graphs give the same bits as the same steps
    launched kernel by kernel (NBODY_GRAPHS=0), over calls that replay a
    captured graph several times: for Barnes-Hut the resident step (one graph
    per buffer parity) and the page-locked host step with its copies, for the
    direct sum the page-locked host call (gather, step, scatter)."""
    torch = cuda
    from nbody_gb300 import initializers as I

    pos, vel, mass = I.plummer(n, a=50.0, seed=5)
    out = {}
    for graphs in ("1", "0"):
        monkeypatch.setenv("NBODY_GRAPHS", graphs)
        s = _system(nb, torch, pos, vel, mass, pinned)
        solver = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode=mode, theta2=0.25)
        for _ in range(3):
            solver.update_particle_positions(s)  # host arrays in and out
        solver.update_particle_positions(s, steps=4)
        solver.upload(s)
        solver.step(5)  # resident steps, both parities replayed
        solver.download(s)
        solver.close()
        out[graphs] = s
    _same(out["1"], out["0"])
