"""Replica sharding and the cross-rank timing reduction, world size 2 over
gloo on the CPU (the multi-GPU bench path without GPUs)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from pmmc_gb300.replicas import combine, shard_seeds


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seeds = list(shard_seeds(rank, world, 64))
        # rank r's step took 100 + 50 r ms and made 1000 (r + 1) moves
        step, moves = combine(100.0 + 50.0 * rank, 1000.0 * (rank + 1))
        out.put((rank, seeds, step, moves))
    finally:
        dist.destroy_process_group()


def test_shards_are_disjoint_and_cover():
    world, per = 4, 64
    allseeds = [s for r in range(world) for s in shard_seeds(r, world, per)]
    assert sorted(allseeds) == list(range(world * per))
    with pytest.raises(ValueError):
        shard_seeds(4, 4, 64)


def test_combine_without_process_group_is_local():
    assert combine(12.5, 7.0) == (12.5, 7.0)


def test_two_rank_gloo_max_and_sum():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, t0, m0), (r1, s1, t1, m1) = got
    assert (r0, r1) == (0, 1)
    assert s0 == list(range(0, 64)) and s1 == list(range(64, 128))
    assert t0 == t1 == 150.0          # the slowest rank
    assert m0 == m1 == 3000.0         # all ranks' moves
