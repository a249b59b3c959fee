"""The tensor-core kernel-matrix build (exact integer distances from fp16
digit planes on tcgen05, fixed-point exponential) against the FP64
dot-product build and the oracle, over the kernel shapes it serves, and its
repeatability: tensor memory is reused tile after tile, so a result must not
depend on what ran before it on the same SMs."""
import os

import numpy as np
import pytest

from oracle import gpr_oracle as O

pytestmark = pytest.mark.gpu


def _problem(n, d, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(1.0, 0.5, size=(n, d))
    X[:, -1] = rng.uniform(-np.pi, np.pi, size=n)
    y = np.sin(X[:, 0]) + 0.3 * np.cos(X[:, -1]) + 1e-3 * rng.normal(size=n)
    return X, y


SPECS = {
    "rbf": lambda d: [O.RBF, d, *range(1, d + 1)],
    "periodic": lambda d: [O.PERIODIC, 2, d - 1, d],
    "rbf_plus_per": lambda d: [O.RBF, d - 1, *range(1, d), O.PERIODIC, 1, d, O.SUM],
    "rbf_times_per_plus_const": lambda d: [O.RBF, d - 1, *range(1, d), O.PERIODIC, 1, d, O.PROD, O.CONSTANT, 0,
                                           O.SUM],
    "const_times_rbf_plus_linear": lambda d: [O.CONSTANT, 0, O.RBF, d, *range(1, d + 1), O.PROD, O.LINEAR, 1, 1,
                                              O.SUM],
}


def _engine(X, y, ks, lik, build):
    from fgpu import Engine
    old = os.environ.get("FGPU_BUILD")
    os.environ["FGPU_BUILD"] = build
    try:
        return Engine(X, y, O.mean_vector("constant", X, y), ks, lik, 1e-6, False)
    finally:
        if old is None:
            del os.environ["FGPU_BUILD"]
        else:
            os.environ["FGPU_BUILD"] = old


@pytest.mark.parametrize("spec", sorted(SPECS))
@pytest.mark.parametrize("n", [77, 300])
def test_tensor_build_matches_fp64_build_and_oracle(spec, n, lib):
    d = 5
    X, y = _problem(n, d, seed=n + len(spec))
    ks = SPECS[spec](d)
    lik = n % 2
    th = np.random.default_rng(3).uniform(0.05, 0.8, size=O.kernel_nparams(ks))
    tc = _engine(X, y, ks, lik, "tc")
    fp = _engine(X, y, ks, lik, "fp64")
    ll_tc, i_tc = tc.loglik(th)
    ll_fp, i_fp = fp.loglik(th)
    ref, rinfo = O.loglik(ks, th, X, y, O.mean_vector("constant", X, y), lik, 1e-6, False)
    assert i_tc == i_fp == rinfo == 0
    assert abs(ll_tc - ref) <= 1e-9 * abs(ref), (ll_tc, ref)
    assert abs(ll_tc - ll_fp) <= 2e-9 * abs(ref), (ll_tc, ll_fp)


def test_tensor_build_is_repeatable_after_other_work(lib):
    from fgpu import loglik_batch
    X, y = _problem(1000, 6, seed=1)
    ks = SPECS["rbf_plus_per"](6)
    e = _engine(X, y, ks, 0, "tc")
    th = np.array([0.2, 0.4, 0.1, 0.3, 0.5, 0.7])
    first, _ = e.loglik(th)
    # other tiles through the same tensor memory: another kernel shape and size
    X2, y2 = _problem(700, 4, seed=2)
    other = _engine(X2, y2, SPECS["rbf_times_per_plus_const"](4), 1, "tc")
    loglik_batch([other] * 8, [np.array([0.3, 0.2, 0.6, 0.9, 0.1])] * 8)
    again, _ = e.loglik(th)
    batched, _ = loglik_batch([e] * 5, [th] * 5)
    assert again == first
    assert np.all(batched == first)
