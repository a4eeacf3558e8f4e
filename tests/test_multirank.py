"""bench.py's multi-GPU arithmetic on CPU: two gloo ranks, each timing its
own replica; the job value uses the slowest rank (replicas only: the path
has no exchange step)."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 + 50.0 * rank          # rank 1 is the slower replica
    slowest = bench.reduce_max(local_ms, dist, "cpu")
    value = bench.replica_throughput(world, 1_000_000, 10, slowest)
    out.put((rank, slowest, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_use_the_slowest_replica():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    results = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slowest, value in results:
        assert slowest == 150.0
        # 2 replicas x 1e6 particles x 2 substeps x 10 steps in 0.15 s
        assert value == pytest.approx(2 * 1_000_000 * 2 * 10 / 0.150)


def test_single_process_is_identity():
    import bench
    assert bench.reduce_max(12.5, None, "cpu") == 12.5
    assert bench.replica_throughput(1, 1000, 4, 2.0) == pytest.approx(1000 * 2 * 4 / 0.002)
