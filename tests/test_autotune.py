"""The autotuner's host logic with a fake timer (no GPU): it picks the
fastest candidate per shape, caches the choice by shape key, samples the
largest problems, never picks a candidate that failed to run, and saves its
cache safely from several processes at once."""
import json
import multiprocessing as mp
import os
import sys

import numpy as np
import pytest

from fgpu import autotune as A


def wl(n, d=3, particles=4, kspec=None):
    rng = np.random.default_rng(n)
    X = rng.normal(size=(n, d))
    y = rng.normal(size=n)
    return A.Workload(X, y, np.zeros(n), kspec or [1, d] + list(range(1, d + 1)), 0, 1e-8, False, particles)


class FakeTimer:
    def __init__(self, ms):
        self.ms, self.calls = ms, []

    def __call__(self, cfg, sample):
        self.calls.append((cfg.name, sum(w.particles for w in sample)))
        v = self.ms[cfg.name]
        if v is None:
            raise RuntimeError("cannot run")
        return v / 1e3


def test_picks_the_fastest_and_caches_by_shape(tmp_path):
    cache = A.TuneCache(str(tmp_path / "t.json"))
    t = FakeTimer({"tcgen05/tc": 5.0, "tcgen05/fp64": 3.0, "fp64/fp64": 9.0})
    cfg, ms, hit = A.tune([wl(500)], timer=t, cache=cache, device="gb300", sms=152)
    assert cfg == A.Config("tcgen05", "fp64") and not hit and len(t.calls) == 3
    assert ms == {"tcgen05/tc": 5.0, "tcgen05/fp64": 3.0, "fp64/fp64": 9.0}
    # same shape (N in the same power-of-two bucket): from the cache, no timing
    cfg2, _, hit2 = A.tune([wl(400)], timer=t, cache=A.TuneCache(str(tmp_path / "t.json")), device="gb300",
                           sms=152)
    assert hit2 and cfg2 == cfg and len(t.calls) == 3
    # another shape is timed again
    t.ms["tcgen05/tc"] = 1.0
    cfg3, _, hit3 = A.tune([wl(4000)], timer=t, cache=cache, device="gb300", sms=152)
    assert not hit3 and cfg3 == A.DEFAULT and len(t.calls) == 6


def test_failed_candidates_are_never_chosen(tmp_path):
    cache = A.TuneCache(str(tmp_path / "t.json"))
    t = FakeTimer({"tcgen05/tc": None, "tcgen05/fp64": 7.0, "fp64/fp64": 8.0})
    cfg, ms, _ = A.tune([wl(300)], timer=t, cache=cache)
    assert cfg.name == "tcgen05/fp64" and ms["tcgen05/tc"] == float("inf")
    t2 = FakeTimer({"tcgen05/tc": None, "tcgen05/fp64": None, "fp64/fp64": None})
    cfg2, _, _ = A.tune([wl(70)], timer=t2, cache=cache, retune=True)
    assert cfg2 == A.DEFAULT


def test_sample_takes_the_largest_problems_first():
    batch = [wl(500, particles=30), wl(6000, particles=30), wl(3000, particles=30)]
    s = A.sample_batch(batch, max_problems=8)
    assert [w.N for w in s] == [6000] and s[0].particles == 8
    s2 = A.sample_batch([wl(500, particles=3), wl(6000, particles=2), wl(3000, particles=2)], max_problems=6)
    assert [(w.N, w.particles) for w in s2] == [(6000, 2), (3000, 2), (500, 2)]


def test_shape_key_buckets():
    k1 = A.shape_key([wl(500)], "gb300", 152)
    assert k1 == A.shape_key([wl(300)], "gb300", 152)       # N 300 and 500 share the 512 bucket
    assert k1 != A.shape_key([wl(600)], "gb300", 152)
    assert k1 != A.shape_key([wl(500, d=4)], "gb300", 152)
    assert k1 != A.shape_key([wl(500)], "gb200", 152)
    assert k1 != A.shape_key([wl(500, particles=40)], "gb300", 152)


def test_config_names_round_trip():
    for c in A.CANDIDATES:
        assert A.Config.from_name(c.name) == c



PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "ferebus-v7_gb300")


def _put_many(path, rank, n):
    sys.path.insert(0, PKG)
    from fgpu import autotune as A2
    for k in range(n):
        A2.TuneCache(path).put(f"rank{rank}-{k}", A2.Config.from_name("tcgen05/tc"), {"tcgen05/tc": 1.0})


def test_ranks_saving_the_cache_at_once(tmp_path):
    """Several processes (the ranks of one job, tuning on a fresh machine at
    the same time) save the cache concurrently: none fails, and the file is
    always one whole JSON document."""
    path = str(tmp_path / "tune.json")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_put_many, args=(path, r, 40)) for r in range(4)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert [p.exitcode for p in procs] == [0, 0, 0, 0]
    with open(path) as f:
        data = json.load(f)
    assert data and all(v["choice"] == "tcgen05/tc" for v in data.values())
    assert not [n for n in os.listdir(tmp_path) if n.endswith(".tmp")]
