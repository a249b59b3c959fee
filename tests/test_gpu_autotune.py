"""The autotuner on the GPU: every candidate configuration runs and gives
the oracle's likelihood; the tuner's choice is cached per shape; a tuned
swarm evaluates with the chosen configuration."""
import numpy as np
import pytest

from oracle import gpr_oracle as O

pytestmark = pytest.mark.gpu


def _data(n, seed=3):
    rng = np.random.default_rng(seed)
    X = rng.normal(2.0, 0.3, size=(n, 4))
    X[:, -1] = rng.uniform(-np.pi, np.pi, size=n)
    y = np.cos(X[:, 0]) + 0.2 * np.sin(X[:, -1]) + 1e-3 * rng.normal(size=n)
    ks = [O.RBF, 3, 1, 2, 3, O.PERIODIC, 1, 4, O.SUM]
    return X, y, O.mean_vector("constant", X, y), ks


@pytest.mark.parametrize("cfg", ["tcgen05/tc", "tcgen05/fp64", "fp64/fp64"])
def test_every_candidate_gives_the_oracle_likelihood(cfg, lib):
    from fgpu import Engine, Plan, autotune
    X, y, mu, ks = _data(300)
    with autotune.use(autotune.Config.from_name(cfg)):
        e = Engine(X, y, mu, ks, 0, 1e-6, False)
    th = np.array([0.3, 0.6, 0.2, 0.5])
    ll, info = Plan([e, e]).run([th, th * 1.1])
    for k, t in enumerate([th, th * 1.1]):
        ref, rinfo = O.loglik(ks, t, X, y, mu, 0, 1e-6, False)
        assert info[k] == rinfo == 0 and abs(ll[k] - ref) <= 1e-9 * abs(ref), (cfg, k)


def test_tuner_times_candidates_and_caches(lib, tmp_path):
    from fgpu import autotune
    X, y, mu, ks = _data(500, seed=5)
    wl = [autotune.Workload(X, y, mu, ks, 0, 1e-6, False, particles=8)]
    cache = autotune.TuneCache(str(tmp_path / "tune.json"))
    cfg, ms, hit = autotune.tune(wl, cache=cache, device="test", sms=1)
    assert not hit and set(ms) == {c.name for c in autotune.CANDIDATES}
    assert all(np.isfinite(v) and v > 0 for v in ms.values())
    assert ms[cfg.name] == min(ms.values())
    cfg2, _, hit2 = autotune.tune(wl, cache=autotune.TuneCache(str(tmp_path / "tune.json")), device="test", sms=1)
    assert hit2 and cfg2 == cfg


def test_tuned_swarm_runs(lib, tmp_path, monkeypatch):
    from fgpu import Engine
    from fgpu.pso import LockstepPSO, SwarmConfig
    monkeypatch.setenv("FGPU_TUNE_CACHE", str(tmp_path / "tune.json"))
    X, y, mu, ks = _data(260, seed=9)
    e = Engine(X, y, mu, ks, 0, 1e-6, False)
    pso = LockstepPSO([(e, np.zeros(4), np.ones(4))], SwarmConfig(swarm_size=6, iterations=3), seed=2, tune=True)
    (x, cost), = pso.run()
    assert pso.tuned is not None and np.isfinite(cost)
    ll, info = pso.engines[0].loglik(x)
    assert info == 0 and abs(-ll - cost) <= 1e-12 * abs(cost)
