"""Multi-rank bench logic on CPU (gloo, world size 2): replicas only.

Each rank tracks its own seeded trajectory (no data-path collective); the only
cross-rank step is the max of the timed region, and the job throughput counts
every rank's frames over the slowest rank's time.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank
    mx = bench.max_over_ranks(ms, world, "cpu")
    q.put((rank, bench.rank_seed(rank), mx, bench.job_throughput(world, 300, 5, mx)))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time_and_distinct_seeds():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res[0][1] != res[1][1]
    assert res[0][2] == res[1][2] == 150.0
    assert abs(res[0][3] - 2 * 300 * 5 / 0.150) < 1e-6


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
    assert bench.job_throughput(1, 300, 5, 1000.0) == 1500.0
