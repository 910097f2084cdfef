"""Host logic of the multi-GPU path: independent replica sets, no data-path
collective.  Each rank advances its own replicas; the job's throughput is the
units all ranks processed over the slowest rank's time (weak scaling)."""
from __future__ import annotations


def replica_range(n_replicas: int, rank: int, world: int) -> range:
    """Contiguous share of a replica list for one rank (sizes differ by <= 1)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n_replicas, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def job_throughput(units: float, seconds: float, dist=None, device=None) -> tuple[float, float, float]:
    """(job units/s, total units, max seconds over ranks).  `dist` is
    torch.distributed (any backend) or None for one process."""
    if dist is None:
        return units / seconds, units, seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()) / float(t.item()), float(u.item()), float(t.item())
