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
* ``train_sharded``: the multi-atom training run over ranks: each rank
  trains the atoms LPT gives it with a lockstep PSO (one batch plan for its
  atoms' swarms per iteration), every swarm with its own random stream
  seeded by the atom's index, and the per-atom results are all-gathered at
  the end.  The result does not depend on the number of ranks.  This replaces
  the reference's loop over atoms (app/main.f90:78-130) around the swarm
  optimiser (src/optimiser/pso/pso.f90:382-472), which trains one atom
  after the other on one node.
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


def train_sharded(problems, config, seed=17, evaluate_for=None, group=None, sizes=None):
    """Train every problem (atom / property) on the ranks of ``group``.

    problems: list of ``(engine, search_min, search_max)`` as for
    ``fgpu.pso.LockstepPSO``; sizes: N per problem for the partition
    (default: each engine's N); evaluate_for(indices) -> the batch evaluator
    of the rank's problems (default: the engines' batch plan).  Returns on
    every rank {problem index: {"theta", "cost", "evaluations", "failures",
    "rank"}}.  Swarm a draws its random numbers from ``seed + a`` alone.
    """
    import torch.distributed as dist
    from .pso import LockstepPSO
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    if sizes is None:
        sizes = [p[0].N for p in problems]
    mine = lpt_partition(sizes, world)[rank]
    local = {}
    if mine:
        sub = [problems[i] for i in mine]
        ev = evaluate_for(mine) if evaluate_for is not None else None
        pso = LockstepPSO(sub, config, seeds=[seed + i for i in mine], evaluate=ev)
        for i, (x, c), st in zip(mine, pso.run(), pso.states):
            local[i] = {"theta": [float(v) for v in x], "cost": float(c), "evaluations": int(st.evaluations),
                        "failures": int(st.failures), "rank": rank}
    return allgather_results(local, group=group)
