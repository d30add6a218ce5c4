"""Replica host logic of bench.py on CPU: two gloo ranks, max-over-ranks
timing and the whole-job aggregate (the path runs as independent replicas
with no data-path collective)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.env_rank()[:2] == (rank, world)
        ms = 10.0 + 7.5 * rank  # the second replica is slower
        t = bench.replica_time_ms(ms, dist)
        dist.barrier()
        q.put((rank, t, bench.job_rate(world, 512.0 ** 3, 200, t)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _ in out] == [17.5, 17.5]
    assert out[0][2] == pytest.approx(2 * 512 ** 3 * 200 / 17.5e-3)


def test_single_process_needs_no_collective():
    import bench

    assert bench.replica_time_ms(3.25, None) == 3.25
    assert bench.job_rate(1, 8.0, 4, 2.0) == pytest.approx(16000.0)
