"""Sharding of independent GPR problems across GPUs (one process per GPU).

Problems (atom x property x particle) are independent, so they shard with no
data-path collective: each rank owns whole problems, evaluates them with its
own engine plans, and the only exchange is a per-iteration all-gather of a few
numbers per problem (cost, info, and the swarm's best position), which can go
through the host.

* ``lpt_partition``: longest-processing-time-first assignment by the
  Cholesky cost N^3 (problems sorted by decreasing cost, each given to the
  least-loaded rank); deterministic for equal costs (lower index first).
* ``allgather_results``: one ``torch.distributed.all_gather_object`` of the
  rank's {problem index: result}; every rank returns the merged dict.
* ``global_best``: reduce per-rank (cost, position) of one shared swarm to
  the swarm's global best, ties broken by the lowest rank (particle order).
"""
from __future__ import annotations

import heapq


def lpt_partition(sizes, nranks):
    """sizes: N per problem -> list of problem-index lists, one per rank."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-float(sizes[i]) ** 3, i))
    heap = [(0.0, r) for r in range(nranks)]
    heapq.heapify(heap)
    out = [[] for _ in range(nranks)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(sizes[i]) ** 3, r))
    return [sorted(x) for x in out]


def loads(sizes, parts):
    return [sum(float(sizes[i]) ** 3 for i in p) for p in parts]


def allgather_results(local, group=None):
    """local: {problem index: result} -> merged dict over all ranks."""
    import torch.distributed as dist
    ws = dist.get_world_size(group)
    bucket = [None] * ws
    dist.all_gather_object(bucket, local, group=group)
    merged = {}
    for part in bucket:
        overlap = set(merged) & set(part)
        if overlap:
            raise RuntimeError(f"problems {sorted(overlap)} owned by two ranks")
        merged.update(part)
    return merged


def global_best(cost, position, group=None):
    """Best (lowest) cost over ranks; ties go to the lowest rank."""
    import torch.distributed as dist
    ws = dist.get_world_size(group)
    bucket = [None] * ws
    dist.all_gather_object(bucket, (float(cost), list(map(float, position))), group=group)
    best_rank = min(range(ws), key=lambda r: (bucket[r][0], r))
    return bucket[best_rank][0], bucket[best_rank][1], best_rank
