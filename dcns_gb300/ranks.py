"""Host-side logic of multi-process runs (one process per GPU, launched by torchrun).

Pairs are independent, so the path shards without any data exchange: rank r aligns its own batch (weak scaling),
and the only collectives are the barrier around the timed region and the max over ranks of the elapsed time.
"""
from __future__ import annotations

BASE_SEED = 20261205


def shard_seed(rank: int) -> int:
    """Seed of rank `rank`'s synthetic batch: every rank draws a different batch of the same distribution."""
    return BASE_SEED + rank


def max_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    """The maximum of `value` over all ranks (the slowest rank bounds a weak-scaling step); `value` when alone."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    """The sum of `value` over all ranks (work done by the whole job); `value` when alone."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, max_ms: float) -> float:
    """Units per second of the whole job: every rank processed `units_per_rank` within `max_ms` milliseconds."""
    return world * units_per_rank / (max_ms * 1e-3)
