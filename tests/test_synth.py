"""The seeded synthetic training sets that stand in for the five benchmark
configurations (fgpu/synth.py), on the CPU: sizes, kernel specs, likelihood
and mean, swarm shapes, feature distributions, the parameter search boxes
and determinism."""
import numpy as np
import pytest

from fgpu import synth
from fgpu.kernel_spec import PERIODIC, RBF, SUM, nparams, parse_kspec


def _leaves(spec):
    return [(n[1], [d + 1 for d in n[2]]) for n in parse_kspec(spec) if n[0] == "leaf"]


def test_water_like():
    p = synth.config1()
    assert (p.N, p.d) == (500, 3)
    assert p.kspec == [RBF, 2, 1, 2, PERIODIC, 1, 3, SUM]
    assert (p.likelihood, p.mean, p.noise, p.optimise_noise) == (0, "constant", 1e-10, False)
    assert (p.swarm, p.iterations) == (20, 50)
    np.testing.assert_allclose(p.X.mean(axis=0), [1.81, 1.81, 1.82], atol=0.01)
    np.testing.assert_allclose(p.X.std(axis=0), [0.05, 0.05, 0.08], rtol=0.1)


def test_methanol_like():
    p = synth.config2()
    assert (p.N, p.d) == (2000, 12)
    assert _leaves(p.kspec) == [(RBF, list(range(1, 10))), (PERIODIC, [10, 11, 12])]
    assert (p.likelihood, p.mean, p.swarm, p.iterations) == (0, "constant", 50, 100)
    assert np.all(np.abs(p.X[:, 9:]) <= np.pi)
    assert np.all((p.X[:, 6:9] >= 1.7) & (p.X[:, 6:9] <= 2.1))


def test_glycine_like():
    p = synth.config3()
    assert (p.N, p.d) == (4000, 24)
    dih = list(range(6, 25, 3))
    assert len(dih) == 7
    assert _leaves(p.kspec) == [(RBF, [f for f in range(1, 25) if f not in dih]), (PERIODIC, dih)]
    assert nparams(p.kspec) == p.ntheta == 24
    assert (p.likelihood, p.swarm, p.iterations) == (1, 40, 100)
    for f in dih:
        assert np.all(np.abs(p.X[:, f - 1]) <= np.pi)
    rest = [f - 1 for f in range(1, 25) if f not in dih]
    assert abs(p.X[:, rest].mean() - 2.2) < 0.01 and abs(p.X[:, rest].std() - 0.15) < 0.01


def test_ragged_atoms():
    atoms = synth.config4()
    assert len(atoms) == 33
    sizes = [a.N for a in atoms]
    assert min(sizes) >= 500 and max(sizes) <= 6000 and len(set(sizes)) > 20
    dih = list(range(6, 94, 3))
    assert len(dih) == 30
    for a in atoms:
        assert a.d == 93 and (a.mean, a.likelihood, a.swarm, a.iterations) == ("linear", 0, 30, 60)
        assert _leaves(a.kspec)[1] == (PERIODIC, dih)
    small = synth.config4(scale=0.05)
    assert [a.N for a in small] == [max(2, int(round(n * 0.05))) for n in sizes]


def test_large_n_with_optimised_noise():
    p = synth.config5()
    assert (p.N, p.d) == (10000, 30)
    assert (p.mean, p.likelihood, p.optimise_noise, p.swarm, p.iterations) == ("quadratic", 0, True, 16, 40)
    assert p.ntheta == nparams(p.kspec) + 1 == 31
    th = p.thetas(500)
    assert th.shape == (500, 31)
    assert np.all((th[:, :-1] >= 1e-3) & (th[:, :-1] <= 1.0))
    # the noise parameter is linear in the reference's box [1e-12, 1e-6],
    # log-uniform across it
    assert np.all((th[:, -1] >= 1e-12) & (th[:, -1] <= 1e-6))
    lg = np.log10(th[:, -1])
    assert lg.min() < -11.5 and lg.max() > -6.5


@pytest.mark.parametrize("make", [synth.config1, synth.config3])
def test_seeded_and_deterministic(make):
    a, b = make(), make()
    assert np.array_equal(a.X, b.X) and np.array_equal(a.y, b.y)
    assert np.array_equal(a.thetas(8, seed=2), b.thetas(8, seed=2))
    assert not np.array_equal(a.thetas(8, seed=2), a.thetas(8, seed=3))
