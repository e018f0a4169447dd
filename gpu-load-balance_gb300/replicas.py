"""Whole-job numbers of N independent replicas (one process per GPU, torchrun).

The ORB path does not shard across GPUs on this hardware (one GPU per box), so N GPUs run N
independent builds. The job's time is the slowest rank's, its work the sum over ranks.
"""
from __future__ import annotations


def whole_job(local_ms: float, local_units: int):
    """Returns (max_ms over ranks, total units over ranks, units per second of the job)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return local_ms, local_units, local_units / (local_ms / 1e3)
    t = torch.tensor([float(local_ms)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([int(local_units)], dtype=torch.int64)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    ms, units = float(t.item()), int(u.item())
    return ms, units, units / (ms / 1e3)
