"""The lockstep PSO driver on the engine: one batched evaluation per iteration
for a swarm, and for several atoms' swarms at once."""
import numpy as np
import pytest

from oracle import gpr_oracle as O

pytestmark = pytest.mark.gpu


def test_single_swarm_water_like(lib):
    from fgpu import Engine, synth
    from fgpu.pso import LockstepPSO, SwarmConfig
    p = synth.config1(200)
    mu = O.mean_vector(p.mean, p.X, p.y)
    e = Engine(p.X, p.y, mu, p.kspec, p.likelihood, p.noise, False)
    lo, hi = np.full(e.ntheta, 1e-3), np.ones(e.ntheta)
    pso = LockstepPSO([(e, lo, hi)], SwarmConfig(swarm_size=20, iterations=6), seed=1)
    (x, cost), = pso.run()
    h = np.array(pso.states[0].history)
    assert np.all(np.diff(h) <= 0) and np.isfinite(cost)
    ll, info = e.loglik(x)
    assert info == 0 and abs(-ll - cost) <= 1e-9 * abs(cost)


def test_multi_atom_lockstep_ragged(lib):
    from fgpu import Engine, synth
    from fgpu.pso import LockstepPSO, SwarmConfig
    atoms = synth.config4(natoms=3, nmin=90, nmax=260)
    probs = []
    for a in atoms:
        mu = O.mean_vector(a.mean, a.X, a.y)
        e = Engine(a.X, a.y, mu, a.kspec, a.likelihood, a.noise, False)
        probs.append((e, np.zeros(e.ntheta), np.ones(e.ntheta)))
    pso = LockstepPSO(probs, SwarmConfig(swarm_size=8, iterations=4), seed=2)
    res = pso.run()
    for (x, cost), (e, _, _) in zip(res, probs):
        ll, info = e.loglik(x)
        assert info == 0 and abs(-ll - cost) <= 1e-9 * abs(cost)


def test_sharded_training_on_the_engine(lib):
    """fgpu.partition.train_sharded on the engine, as one rank of a gloo
    process group: every atom trained with its own random stream gives
    exactly what the lockstep driver gives with the same streams (the
    multi-rank partition itself is tested on the CPU with 2 ranks)."""
    import os
    import socket
    torch = pytest.importorskip("torch")
    import torch.distributed as dist
    from fgpu import Engine, synth
    from fgpu.partition import train_sharded
    from fgpu.pso import LockstepPSO, SwarmConfig
    atoms = synth.config4(natoms=3, nmin=90, nmax=260)
    probs = []
    for a in atoms:
        mu = O.mean_vector(a.mean, a.X, a.y)
        e = Engine(a.X, a.y, mu, a.kspec, a.likelihood, a.noise, False)
        probs.append((e, np.zeros(e.ntheta), np.ones(e.ntheta)))
    cfg = SwarmConfig(swarm_size=6, iterations=3)
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=0, world_size=1)
    try:
        res = train_sharded(probs, cfg, seed=50)
    finally:
        dist.destroy_process_group()
    one = LockstepPSO(probs, cfg, seeds=[50 + i for i in range(len(probs))])
    for i, (x, cost) in enumerate(one.run()):
        assert res[i]["theta"] == [float(v) for v in x] and res[i]["cost"] == float(cost)
        ll, info = probs[i][0].loglik(x)
        assert info == 0 and abs(-ll - cost) <= 1e-9 * abs(cost)
