"""Host-side logic of the multi-process path, on CPU with gloo (world size 2)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from sapien_gb300.sharding import aggregate_throughput, max_across_ranks, shard_bounds


def test_shard_bounds_partition_exactly():
    for n in (0, 1, 7, 16384, 16385):
        for world in (1, 2, 3, 8):
            covered = []
            for r in range(world):
                a, b = shard_bounds(n, r, world)
                assert 0 <= a <= b <= n
                covered.extend(range(a, b))
            assert covered == list(range(n))
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = max_across_ranks(1.0 + rank * 0.5, dist)
        dist.barrier()
        a, b = shard_bounds(16384 * world, rank, world)
        q.put((rank, t, b - a, aggregate_throughput(b - a, world, t)))
    finally:
        dist.destroy_process_group()


def test_gloo_max_reduction_and_aggregate_throughput():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time and the same whole-job throughput
    assert all(r[1] == 1.5 for r in res)
    assert all(r[2] == 16384 for r in res)
    assert all(r[3] == pytest.approx(16384 * 2 / 1.5) for r in res)
