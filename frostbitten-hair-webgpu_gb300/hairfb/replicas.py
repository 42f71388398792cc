"""Replicas: one process per GPU, each rendering its own instances or
sessions.  Frames of different instances share no state, so there is no
data-path collective; ranks only agree on the timing (the slowest rank's
time) before rank 0 reports whole-job throughput."""
from __future__ import annotations


def max_over_ranks(values, dist=None, device: str = "cpu") -> list[float]:
    """Element-wise maximum of `values` over all ranks (identity without a
    process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def job_throughput(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job rate of weak-scaled replicas: every rank processed
    `units_per_rank` units, and the job took the slowest rank's `seconds`."""
    return world * units_per_rank / seconds if seconds > 0 else 0.0
