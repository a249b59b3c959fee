"""Batch plans run in memory-bounded waves.

A plan whose problems' workspaces do not fit the device-memory budget at
once (the 33-atom x 30-particle batch: ~1000 problems of N up to 6000) runs
them in waves that share one workspace arena, all in one graph replay.  The
partition rule is host code and is checked here without a GPU; the GPU test
forces a small budget and checks that the waved plan returns exactly what
one-problem calls return.
"""
import os

import numpy as np
import pytest


def test_everything_fits_is_one_wave_in_caller_order(lib):
    from fgpu.gpr import plan_partition
    wave, n = plan_partition([5, 1, 9, 3], budget=100)
    assert n == 1 and wave == [0, 0, 0, 0]


def test_first_fit_in_decreasing_size(lib):
    from fgpu.gpr import plan_partition
    sizes = [40, 10, 70, 30, 20, 60, 50]
    wave, n = plan_partition(sizes, budget=100)
    # decreasing: 70 60 50 40 30 20 10 -> [70] [60] [50 40] [30 20 10]
    assert n == 4
    assert wave[2] == 0 and wave[5] == 1 and wave[6] == wave[0] == 2
    assert wave[3] == wave[4] == wave[1] == 3
    for w in range(n):
        assert sum(s for s, v in zip(sizes, wave) if v == w) <= 100


def test_random_partitions_respect_the_budget(lib):
    from fgpu.gpr import plan_partition
    rng = np.random.default_rng(4)
    for trial in range(200):
        sizes = rng.integers(1, 1000, size=rng.integers(1, 60))
        budget = int(rng.integers(sizes.max(), sizes.sum() + 2))
        wave, n = plan_partition(sizes, budget)
        assert sorted(set(wave)) == list(range(n))
        for w in range(n):
            assert sum(int(s) for s, v in zip(sizes, wave) if v == w) <= budget
        # waves are filled in decreasing size: no later wave holds a problem
        # larger than any problem of an earlier wave
        if n > 1:
            for w in range(1, n):
                assert max(int(s) for s, v in zip(sizes, wave) if v == w) <= \
                    min(int(s) for s, v in zip(sizes, wave) if v == w - 1)


def test_a_problem_beyond_the_budget_is_an_error(lib):
    from fgpu._lib import FgpuError
    from fgpu.gpr import plan_partition
    with pytest.raises(FgpuError) as e:
        plan_partition([10, 500, 20], budget=100)
    assert e.value.code == -3 and "problem 1" in str(e.value)


@pytest.mark.gpu
def test_waved_plan_equals_plain_calls(lib, monkeypatch):
    """A ragged batch under a budget that forces several waves: every problem's
    ll equals its one-problem call bit for bit, and a replay repeats it."""
    from fgpu import Engine, Plan
    from oracle import gpr_oracle as O
    rng = np.random.default_rng(77)
    engines, thetas = [], []
    for k, (n, lik) in enumerate([(300, 0), (700, 1), (130, 0), (1, 0), (520, 0), (257, 1)]):
        X = rng.normal(2.0, 0.3, size=(n, 4))
        X[:, -1] = rng.uniform(-np.pi, np.pi, size=n)
        y = np.cos(X[:, 0]) + 0.2 * np.sin(X[:, -1]) + 1e-3 * rng.normal(size=n)
        ks = [O.RBF, 3, 1, 2, 3, O.PERIODIC, 1, 4, O.SUM]
        mu = O.mean_vector("constant", X, y)
        engines.append(Engine(X, y, mu, ks, lik, 1e-6, False))
        thetas.append(rng.uniform(0.0, 1.0, size=4))
    probs = [engines[i % 6] for i in range(14)]
    ths = [thetas[i % 6] + 0.01 * (i // 6) for i in range(14)]
    whole = Plan(probs)
    nw1, total = whole.waves()
    assert nw1 == 1
    budget_mb = total / 3.0 / 2 ** 20 + 0.5     # room for about a third of the batch
    monkeypatch.setenv("FGPU_PLAN_MEM_BUDGET_MB", str(budget_mb))
    waved = Plan(probs)
    nw, arena = waved.waves()
    assert nw >= 3 and arena <= budget_mb * 2 ** 20
    ll, info = waved.run(ths)
    ll1, info1 = whole.run(ths)
    for i in range(14):
        l0, i0 = probs[i].loglik(ths[i])
        assert info[i] == info1[i] == i0 == 0
        assert ll[i] == ll1[i] == l0
    ll2, _ = waved.run(ths)
    assert np.array_equal(ll, ll2)
