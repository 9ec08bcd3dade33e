"""Host-side logic of the multi-process path, on CPU with gloo (world size 2)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from sapien_gb300.sharding import aggregate_throughput, max_across_ranks, shard_bounds, sum_across_ranks


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


def _rollout_problem(n=48, T=25):
    """A small instance of the differentiable-rollout workload (9-DoF arm, semi-implicit
    Euler at dt = 1/500, tau ~ N(0, 5) per step, loss = summed squared end-effector
    distance to seeded targets)."""
    import numpy as np

    from sapien_gb300 import synthetic as syn

    robot = syn.arm_with_fingers()
    q0, qd0, _, _ = robot.sample(n, seed=13)
    rng = np.random.default_rng(14)
    tau = rng.normal(scale=5.0, size=(T, n, robot.nv))
    targets = rng.uniform(-0.5, 0.5, size=(n, 3))
    return robot, q0, qd0, tau, targets


def _oracle(robot):
    from oracle.oracle import Oracle

    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    return o


def _shard_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        robot, q0, qd0, tau, targets = _rollout_problem()
        a, b = shard_bounds(q0.shape[0], rank, world)
        qT, qdT, loss = _oracle(robot).rollout(q0[a:b], qd0[a:b], tau[:, a:b], 1.0 / 500, robot.ee_link, targets[a:b])
        total = sum_across_ranks(float(loss.sum()), dist)
        q.put((rank, a, b, qT, qdT, total))
    finally:
        dist.destroy_process_group()


def test_sharded_rollout_loss_equals_single_process():
    """Each gloo rank rolls out its own shard of environments (no data-path exchange); the
    per-shard losses summed on the host equal the single-process loss, and every rank's
    final states equal the single-process rows."""
    import numpy as np

    world = 2
    ctx = mp.get_context("spawn")
    qu = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, world, port, qu)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((qu.get(timeout=180) for _ in range(world)), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    robot, q0, qd0, tau, targets = _rollout_problem()
    qT, qdT, loss = _oracle(robot).rollout(q0, qd0, tau, 1.0 / 500, robot.ee_link, targets)
    for rank, a, b, qTs, qdTs, total in res:
        assert np.array_equal(qTs, qT[a:b]) and np.array_equal(qdTs, qdT[a:b])
        assert total == pytest.approx(float(loss.sum()), rel=1e-13)
    assert res[0][2] == res[1][1]  # shards are contiguous and cover everything
