"""Multi-GPU runs of the solver: independent replicas, one process per GPU.

The reference's only multi-GPU use maps MPI rank -> GPU with no messages
(PASIf.py:27-30, :167); systems are independent, so N GPUs run N replicas of a
sweep (weak scaling) and the only collective is the max-over-ranks of the
timed region, outside the data path.
"""
from __future__ import annotations


def max_over_ranks(x: float, dist=None, device: str = "cpu") -> float:
    """Maximum of x over the ranks of the default process group (x itself
    without one)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, world: int, slowest_seconds: float) -> float:
    """Whole-job throughput: the units every rank processed over the slowest
    rank's time."""
    return world * units_per_rank / slowest_seconds
