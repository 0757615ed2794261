"""Independent work across ranks (one process per GPU): ensemble slices and whole-simulation
replicas.

Ranks that run independent simulations (or slices of an ensemble, split by instance) combine
only their timings and work counts: the job-wide rate is the total work of all ranks over the
slowest rank's time. One simulation sharded over ranks is phasefield_gb300/sharding.py.
"""
from __future__ import annotations


def aggregate(local_ms: float, local_updates: int, dist=None, device=None) -> tuple[float, int]:
    """Returns (max time over ranks in ms, total updates over ranks)."""
    if dist is None or not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(local_ms), int(local_updates)
    import torch
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    w = torch.tensor([float(local_updates)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), int(round(w.item()))


def split_instances(n_instances: int, rank: int, world: int) -> range:
    """Contiguous slice of an ensemble owned by `rank` (instances are independent)."""
    per, rem = divmod(n_instances, world)
    start = rank * per + min(rank, rem)
    return range(start, start + per + (1 if rank < rem else 0))
