"""Independent replicas over ranks: the multi-GPU mode of this path.

Homogenization solves are independent, so N GPUs run N replicas with no exchange on
the data path: each rank takes its share of the work (solves, requests), times it on
its own device, and the job's throughput is all units over the slowest rank's time
(max over ranks), the only collective being that one reduction at the end.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple


def shard(items: Sequence, rank: int, world: int) -> List:
    """Round-robin share of items for rank (item i goes to rank i mod world)."""
    return [x for i, x in enumerate(items) if i % world == rank]


def aggregate_throughput(units: float, seconds: float, group=None) -> Tuple[float, float, float]:
    """(whole-job units per second, max seconds over ranks, total units) from this
    rank's units and elapsed seconds.  With torch.distributed initialised this is two
    all-reduces (max of the time, sum of the units); otherwise the local values."""
    try:
        import torch
        import torch.distributed as dist
        active = dist.is_available() and dist.is_initialized()
    except ImportError:
        active = False
    if not active:
        return (units / seconds if seconds > 0 else 0.0), seconds, units
    dev = 'cuda' if dist.get_backend(group) == 'nccl' else 'cpu'
    t = torch.tensor([seconds], dtype=torch.float64, device=dev)
    u = torch.tensor([units], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    tmax, utot = float(t.item()), float(u.item())
    return (utot / tmax if tmax > 0 else 0.0), tmax, utot
