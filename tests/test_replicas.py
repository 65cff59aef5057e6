"""Replica bookkeeping over two gloo ranks on the CPU: the multi-GPU path is
independent replicas, so these are the only cross-rank steps."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from cpim_gb300.replicas import job_rate, shard


def test_shard_covers_every_item_once():
    for n in (0, 1, 7, 64, 1001):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in shard(n, r, world)]
            assert got == list(range(n))
            sizes = [len(shard(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(5, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        items = shard(10, rank, world)
        units, secs, rate = job_rate(len(items) * 100.0, 1.0 + rank)
        q.put((rank, list(items), units, secs, rate))
    finally:
        dist.destroy_process_group()


def test_job_rate_two_gloo_ranks():
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
    assert [o[1] for o in out] == [[0, 1, 2, 3, 4], [5, 6, 7, 8, 9]]
    for _, _, units, secs, rate in out:
        assert units == 1000.0  # 10 items x 100 units, summed over ranks
        assert secs == 2.0      # the slower rank bounds the job
        assert rate == 500.0


def test_job_rate_without_a_process_group():
    assert job_rate(30.0, 2.0) == (30.0, 2.0, 15.0)
