"""Weak-scaling replicas across GPUs (one process per GPU, no data-path
collective): the frames / ROIs of an analysis are independent, as the
reference's parfor over frame blocks (RJ.m:217-244) treats them.  Each rank
works on its own shard; the only exchange is the maximum of the ranks'
timings (and a final gather where a caller wants the results on one rank).
"""
from __future__ import annotations


def shard(n_units: int, rank: int, world: int) -> range:
    """Contiguous share of units 0..n_units-1 for `rank` of `world`
    (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    q, r = divmod(int(n_units), int(world))
    lo = rank * q + min(rank, r)
    return range(lo, lo + q + (1 if rank < r else 0))


def rank_seed(base: int, rank: int) -> int:
    """Workload seed of a rank: every rank draws its own synthetic shard."""
    return int(base) + int(rank)


def max_over_ranks(x: float, dist=None, device: str = "cpu") -> float:
    """The largest of the ranks' values (the slowest rank sets the time);
    x itself without a process group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, world: int, seconds_max: float) -> float:
    """Units of all ranks over the slowest rank's time."""
    return float(world) * float(units_per_rank) / float(seconds_max)
