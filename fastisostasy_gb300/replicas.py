"""Process-level sharding of independent domains (one process per GPU).

LV-ELVA domains do not share cells: every RHS holds a global 2-D transform
of its own domain, so one domain is never split across GPUs.  Ensemble
members and serving requests are independent and shard by member; the only
exchange the reference has between domains is the scalar barystatic volume
change summed over the domains that share one bsl_class
(src/fastisostasy.f90:766-775), which `sum_over_ranks` provides.  With a
single process every helper is the identity.
"""
from typing import List, Sequence


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def world() -> tuple:
    """(rank, world size) of the current process group, (0, 1) without one."""
    d = _dist()
    return (d.get_rank(), d.get_world_size()) if d else (0, 1)


def shard(costs: Sequence[float], rank: int, size: int) -> List[int]:
    """Indices of the items `rank` owns: greedy longest-first assignment of
    the items' costs (e.g. cells x expected steps) to `size` ranks, so every
    rank gets a similar total.  Deterministic: every rank computes the same
    partition."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * size
    owner = [0] * len(costs)
    for i in order:
        r = min(range(size), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += costs[i]
    return [i for i in range(len(costs)) if owner[i] == rank]


def _reduce(x: float, op: str, device=None) -> float:
    d = _dist()
    if d is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    d.all_reduce(t, op=getattr(d.ReduceOp, op))
    return float(t.item())


def max_over_ranks(x: float, device=None) -> float:
    """The slowest rank's time (timed regions are reported as the maximum)."""
    return _reduce(x, "MAX", device)


def sum_over_ranks(x: float, device=None) -> float:
    """Sum of a per-domain scalar over all ranks, e.g. deltaV_bsl of the
    domains coupled through one barystatic sea level."""
    return _reduce(x, "SUM", device)
