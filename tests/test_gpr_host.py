"""The host mirror of the reference's GPR cost-function interface
(fgpu/gpr.py: GaussianProcessRegressor, IterResult), on the CPU with a
stand-in engine: cost = -logL, success = (info == 0)
(src/optimiser/iter_result.f90:92-101), the noise parameter's box
[1e-12, 1e-6] and its place last in the parameter vector
(src/model/gpr/gpr.f90:221-245), and the weights call."""
import numpy as np
import pytest

from fgpu.gpr import GaussianProcessRegressor, IterResult, mean_vector


class StandInEngine:
    """Records the parameters it is asked for; logL = -sum(theta^2), info 2
    when the first parameter is negative (a failed factorisation)."""

    def __init__(self):
        self.calls = []

    def loglik(self, theta, want_alpha=False):
        th = np.asarray(theta, dtype=np.float64).copy()
        self.calls.append(th)
        info = 2 if th[0] < 0 else 0
        ll = -float(np.sum(th * th)) if info == 0 else float("nan")
        if want_alpha:
            return ll, info, np.arange(3, dtype=np.float64)
        return ll, info


KS = {"k1": {"type": "rbf", "active_dimensions": [1, 2]}, "k2": {"type": "periodic", "active_dimensions": [3]}}


def _gp(**kw):
    X = np.random.default_rng(1).normal(size=(6, 3))
    eng = StandInEngine()
    return GaussianProcessRegressor(X, X[:, 0], "k1*k2", KS, engine=eng, **kw), eng


def test_cost_function_is_minus_loglik_and_success_is_info_zero():
    gp, eng = _gp()
    assert gp.nparams() == 3
    r = gp.cost_function([0.1, 0.2, 0.3])
    assert isinstance(r, IterResult) and r.success and r.info == 0
    assert r.cost == pytest.approx(0.14)
    np.testing.assert_array_equal(eng.calls[-1], [0.1, 0.2, 0.3])
    np.testing.assert_array_equal(gp.get_params(), [0.1, 0.2, 0.3])
    bad = gp.cost_function([-0.1, 0.2, 0.3])
    assert not bad.success and bad.info == 2 and np.isnan(bad.cost)


def test_noise_parameter_is_last_and_boxed():
    gp, eng = _gp(optimise_noise=True, search_min=0.5, search_max=2.0)
    assert gp.nparams() == 4
    np.testing.assert_array_equal(gp.search_min(), [0.5, 0.5, 0.5, 1e-12])
    np.testing.assert_array_equal(gp.search_max(), [2.0, 2.0, 2.0, 1e-6])
    gp.cost_function([1.0, 1.0, 1.0, 3e-9])
    assert gp.nugget == 3e-9
    assert eng.calls[-1][-1] == 3e-9  # the engine gets the linear noise value itself


def test_parameter_count_is_checked():
    gp, _ = _gp()
    with pytest.raises(ValueError):
        gp.set_params([0.1, 0.2])


def test_weights_come_from_the_engine():
    gp, eng = _gp()
    gp.set_params([0.1, 0.2, 0.3])
    alpha, info = gp.weights()
    assert info == 0 and alpha.tolist() == [0.0, 1.0, 2.0]


def test_cached_mean_is_the_host_mean_function():
    X = np.random.default_rng(4).normal(size=(20, 3))
    y = X[:, 0] * 2.0 + 1.0
    gp = GaussianProcessRegressor(X, y, "k1", KS, mean="linear", engine=StandInEngine())
    np.testing.assert_allclose(gp.cached_mean, mean_vector("linear", X, y))
    np.testing.assert_allclose(gp.cached_mean, y, atol=1e-10)  # a linear target is its own mean
