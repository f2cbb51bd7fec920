"""Replica aggregation for runs on N GPUs of one node.

The grouped-aggregation path has no exchange step on one GPU, so N GPUs run
N independent replicas (weak scaling: each rank aggregates its own copy of
the workload).  Whole-job throughput is the rows all ranks processed over
the slowest rank's time, taken with one MAX all-reduce outside the timed
region; no collective touches the data path.
"""
from __future__ import annotations


def slowest_ms(local_ms: float, dist=None, device: str = "cpu") -> float:
    """The largest per-step time over all ranks (local_ms when single)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(local_ms)
    import torch

    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rows_per_s(rows_per_rank: int, world: int, slowest_step_ms: float) -> float:
    """Whole-job rows/s: every rank's rows over the slowest rank's step time."""
    return rows_per_rank * world / (slowest_step_ms / 1e3)
