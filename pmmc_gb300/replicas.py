"""Replicas across GPUs: the ensemble shards by structure with no exchange.

Each rank anneals its own structures (independent seeds); the only
cross-rank step is the bench's reduction of its timing and move counts: the
slowest rank's step time and the sum of the moves.  Works with any process
group (nccl on device tensors, gloo on host tensors).
"""
from __future__ import annotations


def shard_seeds(rank: int, world: int, per_rank: int) -> range:
    """Structure seeds of a rank: a contiguous, disjoint block per rank."""
    if not (0 <= rank < world) or per_rank < 0:
        raise ValueError(f"bad shard: rank {rank} of {world}, {per_rank} per rank")
    return range(per_rank * rank, per_rank * (rank + 1))


def combine(step_ms: float, moves: float, device=None) -> tuple[float, float]:
    """(max step time over ranks, total moves over ranks) through the default
    process group; without one, the local values."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(step_ms), float(moves)
    t = torch.tensor([float(step_ms), float(moves)], dtype=torch.float64, device=device)
    got = [torch.zeros_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(got, t)
    return max(float(g[0]) for g in got), sum(float(g[1]) for g in got)
