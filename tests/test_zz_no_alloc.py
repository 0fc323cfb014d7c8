"""nbody_pp_forces_noalloc: the direct-sum entry point for callers that cannot
let a library allocate device memory (a loop that must not stall on
cudaMalloc/cudaFree, or an application whose own pool owns all device memory).
Its scratch is a fixed array inside the library; the caller passes only input
and output buffers.

It is called through the C ABI twice in a row and compared with the
allocating entry point (nbody_pp_forces_device) within the direct-sum force
tolerance used by the other GPU tests: per-body relative error RMS <= 1e-5,
max <= 1e-3, up to 262,144 bodies. At the 4,194,304-body cap the two plans
sum 4M terms per body in different orders and groupings (one FP32 sum per
body here, partial sums there), so they differ by the FP32 accumulation
error, which grows like sqrt(N): there the bound is 1e-5 * sqrt(N / 16,384),
and both are checked against an FP64 direct sum on sampled bodies. This
file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err_stats

pytestmark = pytest.mark.gpu


def _check(got, ref, n):
    rms, mx = rel_err_stats(got, ref)
    scale = (n / 16384) ** 0.5 if n > 262144 else 1.0
    assert rms <= 1e-5 * scale and mx <= 1e-3, (rms, mx)


# Sizes chosen for the plan the fixed 8 MiB array leaves (GB300, 152 SMs):
#   16,384 / 5,000: j-slices whose partial sums fit as planned;
#   131,072: the linear split, whose partials (5 MB) fit;
#   262,144: the linear partials (10 MB) do not fit, the plan falls back to
#            j-slices and cuts them to one;
#   4,194,304: the largest size accepted, one slice;
#   16,384 with NBODY_PP_SLICES=64: 16 MiB of slices, lowered to 31 to fit.
CASES = [(16384, None), (5000, None), (131072, None), (262144, None), (4194304, None), (16384, "64")]


@pytest.mark.parametrize("n,slices", CASES)
def test_noalloc_matches_allocating_entry_point_twice(nb, cuda, oracle, monkeypatch, n, slices):
    torch = cuda
    from nbody_gb300 import initializers as I

    pos, vel, mass = I.uniform_ball(n, seed=77 + n)
    pm = torch.from_numpy(I.pos_mass(pos, mass)).cuda()
    stream = torch.cuda.Stream()
    ref = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    solver = nb.ParticleSolverCUDA(0.0035, 40.0, n, mode="pp")
    solver.set_stream(stream.cuda_stream)
    solver.pp_forces_device(pm, ref)
    stream.synchronize()
    ref_h = ref.cpu().numpy()
    solver.close()

    if slices is not None:
        monkeypatch.setenv("NBODY_PP_SLICES", slices)
    L = nb.lib()
    outs = []
    for _ in range(2):
        out = torch.full((n, 4), float("nan"), dtype=torch.float32, device="cuda")
        status = ctypes.c_int(-1)
        rc = L.nbody_pp_forces_noalloc(pm.data_ptr(), out.data_ptr(), n, 40.0, stream.cuda_stream,
                                       ctypes.byref(status))
        assert rc == nb.OK, nb.status_string(rc)
        assert status.value == nb.OK
        got = out.cpu().numpy()
        _check(got, ref_h, n)
        assert np.all(got[:, 3] == 0)
        outs.append(got)
    # the shared scratch is cleared on every call: the second call repeats the first
    np.testing.assert_array_equal(outs[0], outs[1])
    if n > 262144:
        idx = np.random.default_rng(3).choice(n, 256, replace=False)
        a64 = oracle.direct_f64(I.pos_mass(pos, mass), mass, 40.0, idx=idx)
        e_alloc = rel_err_stats(ref_h[idx], a64)[0]
        e_noalloc = rel_err_stats(outs[0][idx], a64)[0]
        print(f"n={n}: RMS error vs FP64, allocating {e_alloc:.3g}, without allocation {e_noalloc:.3g}")
        assert e_noalloc <= 1e-4 and e_alloc <= 1e-4, (e_noalloc, e_alloc)


def test_noalloc_rejects_too_many_bodies(nb, cuda):
    L = nb.lib()
    n = 4194304 + 1
    rc = L.nbody_pp_forces_noalloc(16, 16, n, 40.0, None, None)  # rejected before any device work
    assert rc == nb.ERR_CAPACITY
    assert L.nbody_pp_forces_noalloc(None, None, 10, 40.0, None, None) == nb.ERR_ARG
