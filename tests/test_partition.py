"""Multi-GPU sharding logic, exercised with 2 gloo ranks on CPU."""
import os
import socket

import numpy as np
import pytest

from fgpu.partition import allgather_results, global_best, loads, lpt_partition


def test_lpt_assigns_every_problem_once_and_balances():
    rng = np.random.default_rng(4)
    sizes = rng.integers(500, 6001, size=33)          # the 33-atom ragged batch
    for nranks in (1, 2, 4, 8):
        parts = lpt_partition(sizes, nranks)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(33))
        ld = loads(sizes, parts)
        # LPT bound: max load <= 4/3 optimum + one job; check against the mean
        assert max(ld) <= sum(ld) / nranks + max(float(s) ** 3 for s in sizes)


def test_lpt_is_deterministic():
    # largest first to the least-loaded rank, ties to the lower index / rank
    assert lpt_partition([1000, 1000, 1000, 2000], 2) == [[3], [0, 1, 2]]
    assert lpt_partition([5, 5, 5, 5], 2) == [[0, 2], [1, 3]]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = [600, 4000, 2500, 1200, 3300]
    mine = lpt_partition(sizes, world)[rank]
    local = {i: {"cost": float(sizes[i]) * 0.5 + rank, "info": 0} for i in mine}
    merged = allgather_results(local)
    cost, pos, who = global_best(10.0 - rank if rank else 10.0, [rank, rank + 1.0])
    q.put((rank, sorted(merged), cost, pos, who))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_gather_and_global_best():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, keys, cost, pos, who in out:
        assert keys == [0, 1, 2, 3, 4]
        assert cost == 9.0 and pos == [1.0, 2.0] and who == 1
