"""Sharding of scoring jobs across ranks (one process per GPU).

The path shards by sample: samples are independent through both passes, so each rank scores its
own jobs with no collective in the data path (weak scaling).  A job is placed by its work, the
aligned read-bases of its sample, with the longest-processing-time rule: heaviest job first, onto
the rank with the least work so far (ties to the lower rank), which is deterministic on every rank
without communication.  Timing across ranks takes the slowest rank (all_reduce MAX)."""
from __future__ import annotations


def plan(work: list[int] | list[float], world: int) -> list[list[int]]:
    """Job indices per rank; every job on exactly one rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    load = [0.0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += work[i]
    for r in out:
        r.sort()
    return out


def slowest(value: float, group=None) -> float:
    """Maximum of `value` over the ranks of the default process group (itself without one)."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
