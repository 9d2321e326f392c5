"""Replica sharding and the cross-rank timing reduction, world sizes 2 and 3
over gloo on the CPU (the multi-GPU bench path without GPUs)."""
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


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_ranks_max_and_sum(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == list(range(world))
    for r, seeds, step, moves in got:
        assert seeds == list(range(64 * r, 64 * (r + 1)))
        assert step == 100.0 + 50.0 * (world - 1)                     # the slowest rank
        assert moves == 1000.0 * world * (world + 1) / 2              # all ranks' moves
