"""Several GPUs as independent replicas: shots and models are independent
units, so ranks split them with no exchange on the data path.

``shard(costs, world)``  assigns units to ranks, longest first to the least
    loaded rank (LPT; at most 4/3 of the optimal makespan), deterministic.
``gather(obj, pg)``       rank 0 receives every rank's result (a dict merged by
    unit index); the only collective, after the work.
``max_over_ranks(x, pg)`` the slowest rank's time, as the bench reports it.
The process group can be NCCL (GPU) or gloo (CPU); nothing here touches a GPU.
"""
from __future__ import annotations

import heapq


def shard(costs, world):
    """List of unit-index lists, one per rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(o) for o in out]


def gather(results, pg=None):
    """results: {unit index: value} of this rank -> merged dict on rank 0, None elsewhere."""
    import torch.distributed as dist
    if pg is None and not dist.is_initialized():
        return dict(results)
    world = dist.get_world_size(pg)
    rank = dist.get_rank(pg)
    bucket = [None] * world if rank == 0 else None
    dist.gather_object(results, bucket, dst=0, group=pg)
    if rank != 0:
        return None
    merged = {}
    for part in bucket:
        overlap = merged.keys() & part.keys()
        if overlap:
            raise RuntimeError("units %s reported by two ranks" % sorted(overlap)[:5])
        merged.update(part)
    return merged


def max_over_ranks(x, pg=None):
    import torch
    import torch.distributed as dist
    if pg is None and not dist.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=pg)
    return float(t.item())
