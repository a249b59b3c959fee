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


# -- the sharded multi-atom training driver ---------------------------------

_SIZES = [600, 4000, 2500, 1200, 3300, 900]   # N per atom (partition weights)
_NTH = [3, 4, 2, 5, 3, 4]                      # parameters per atom


def _problems():
    return [(None, np.full(n, 0.0), np.full(n, 1.0)) for n in _NTH]


def _evaluate_for(indices):
    """A deterministic stand-in for the engine: logL = -|theta - t_a|^2 with
    a per-atom optimum, and a 'Cholesky failure' (info = 1) in a corner of
    the box so that the retry rule runs."""
    def evaluate(positions):
        S = len(positions) // len(indices)
        ll, info = [], []
        for k, x in enumerate(positions):
            a = indices[k // S]
            t = 0.2 + 0.1 * a + 0.05 * np.arange(len(x))
            ll.append(-float(np.sum((np.asarray(x) - t) ** 2)))
            info.append(1 if x[0] > 0.97 else 0)
        return np.array(ll), np.array(info, dtype=np.int32)
    return evaluate


def _sharded_worker(rank, world, port, q):
    import torch.distributed as dist
    from fgpu.partition import train_sharded
    from fgpu.pso import SwarmConfig
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg = SwarmConfig(swarm_size=6, iterations=12)
    res = train_sharded(_problems(), cfg, seed=100, evaluate_for=_evaluate_for, sizes=_SIZES)
    q.put((rank, res))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_training_matches_one_rank():
    """train_sharded on 2 gloo ranks: every atom trained exactly once, on the
    rank LPT gives it, and the results identical (bit for bit) to one
    process training all atoms with the same per-atom random streams."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from fgpu.pso import LockstepPSO, SwarmConfig
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_sharded_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0] == out[1]
    res = out[0]
    parts = lpt_partition(_SIZES, 2)
    assert sorted(res) == list(range(len(_SIZES)))
    for r, part in enumerate(parts):
        assert all(res[i]["rank"] == r for i in part)
    cfg = SwarmConfig(swarm_size=6, iterations=12)
    allidx = list(range(len(_SIZES)))
    one = LockstepPSO(_problems(), cfg, seeds=[100 + i for i in allidx], evaluate=_evaluate_for(allidx))
    for i, ((x, c), st) in enumerate(zip(one.run(), one.states)):
        assert res[i]["theta"] == [float(v) for v in x] and res[i]["cost"] == float(c)
        assert res[i]["evaluations"] == st.evaluations and res[i]["failures"] == st.failures
    assert sum(r["failures"] for r in res.values()) > 0   # the retry rule ran
