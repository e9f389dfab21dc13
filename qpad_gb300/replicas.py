"""Multi-GPU runs are independent replicas: one simulation per GPU, no data-path collective.

A single quasi-static simulation does not shard (xi slices are strictly sequential and a
radial split would need a distributed tridiagonal solve), so N GPUs run N simulations with
different seeds.  The only communication is host-side: a barrier around the timed region
and the reduction of the timings (max over ranks) and of the work done (sum over ranks).
"""
from __future__ import annotations


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of the replica on `rank` (rank 0 keeps the deck's own seed)."""
    return base_seed + 17 * rank


def reduce_timing(seconds: float, units: float, dist=None):
    """(max seconds over ranks, total units over ranks); plain values without a group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return seconds, units
    import torch
    t = torch.tensor([seconds], dtype=torch.float64)
    u = torch.tensor([units], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
