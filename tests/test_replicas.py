"""Multi-GPU form on the CPU: "replicas only" (the per-step solve does not
shard; N GPUs step N independent copies). World-size-2 gloo process groups on
127.0.0.1 check the bench's whole-job aggregation (units of all ranks over the
slowest rank's time, max-over-ranks timing) and that the reference arm's
other ranks leave quietly.
"""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    w, r, local = bench.dist_env()
    dist = bench.init_dist(w, local)
    try:
        mx = bench.max_over_ranks(dist, float(r + 1))
        rate = bench.replica_rate(dist, units=100.0 * (r + 1), seconds=1.0 + r)
        bench.barrier(dist)
        out.put((r, w, mx, rate))
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregation_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1] and all(w == 2 for _, w, _, _ in res)
    # the max of (1, 2); (100 + 200) units over the slowest rank's 2 s
    assert all(mx == 2.0 for _, _, mx, _ in res)
    assert all(rate == pytest.approx(150.0) for *_, rate in res)


def test_single_process_rate_is_local():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.replica_rate(None, 300.0, 2.0) == 150.0
    assert bench.max_over_ranks(None, 3.5) == 3.5


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "pp"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_committed_profiles_give_the_bench_its_traffic():
    """bench.py reads the per-launch DRAM traffic of its roofline kernels from the
    committed ncu summaries: each must parse to a positive byte count."""
    import bench

    for kernel in ("pp_force", "bh_traverse"):
        t = bench.profile_traffic(kernel)
        assert t is not None and t > 0, kernel
    per_body = bench.profile_value("pp_batch_kernel", "traffic_bytes_per_body")
    assert per_body is not None and per_body > 0
    assert bench.profile_traffic("no_such_kernel") is None
