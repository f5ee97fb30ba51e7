"""Multi-GPU form of the benchmark workloads: independent replicas.

One scene's edit path does not shard (one global dedup table per level), so N
GPUs run N independent replicas, one process per GPU, each on its own seeded
batches; no collective touches the data path.  The only exchange is the
whole-job figure at the end: the slowest rank's time and the work of all
ranks.
"""
from __future__ import annotations


def replica_seed(rank: int, batch: int) -> int:
    """Seed of batch `batch` of rank `rank` (different ranks, different edits)."""
    return 1000 + 100 * rank + batch


def replica_totals(elapsed_ms: float, units: float, device=None):
    """(max over ranks of elapsed_ms, sum over ranks of units); the local
    values when no process group is running."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
