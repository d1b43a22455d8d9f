"""Replica sharding on two CPU ranks (gloo): disjoint, complete shards; the
timing maximum and the result gather that bench.py and the sweep use."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from spsslangevinintegration_gb300.replicas import gather_results, max_over_ranks, shard


def test_shard_is_a_partition():
    for count in (0, 1, 7, 512, 513):
        for world in (1, 2, 3, 8):
            seen = [i for r in range(world) for i in shard(count, world, r)]
            assert seen == list(range(count))
            sizes = [len(shard(count, world, r)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = list(shard(10, world, rank))
    t = max_over_ranks(1.0 + rank)
    res = gather_results([(i, i * i) for i in mine])
    if rank == 0:
        out.put((t, res))
    dist.destroy_process_group()


def test_two_rank_gather_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    t, res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert t == 2.0
    assert res == [(i, i * i) for i in range(10)]
