"""Pins for the CPU oracle (runs without a GPU).

The reference ships no golden vectors and cannot be built here, so the
oracle is pinned by internal consistency: the distance-tensor path against
independent per-pair formulas, LAPACK against a pure-Python Cholesky and an
independent LAPACK (MKL through torch, when present), the profiled mean of the
concentrated likelihood against its optimality condition, and the analytic
gradient against central differences.
"""
import math

import numpy as np
import pytest

from conftest import golden_cases, load_case, parity_tol
from oracle import exact as E
from oracle import gpr_oracle as O


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_reproduces_golden(name):
    c = load_case(name)
    ks = [int(v) for v in c["kspec"]]
    tens = O.Tensors(c["X"], need_cyclic=O.RBF_CYCLIC in ks)
    for k, th in enumerate(c["thetas"]):
        ll, info = O.loglik(ks, th, c["X"], c["y"], c["mu"], int(c["likelihood"]), float(c["noise"]),
                            bool(c["optimise_noise"]), tens=tens)
        assert info == int(c["info"][k])
        if info == 0:
            # the oracle is one FP64 evaluation: within the FP64 bar of the
            # extended-precision value, and (same LAPACK) at its stored value
            assert abs(ll - c["ll_exact"][k]) <= parity_tol(c["ll_exact"][k], c["ll"][k], c["fp64_err"][k])
            assert abs(ll - c["ll"][k]) <= 1e-12 * abs(c["ll"][k])


@pytest.mark.parametrize("name", ["water_O1_rbf_x_per", "syn_c1_water_like", "ammonia_N1_rbf",
                                  "linear_in_composite_conc", "cyclic_rbf_all_dims", "composite_prod_sum"])
def test_extended_precision_value_is_far_below_the_fp64_error(name):
    """The extended-precision likelihood (stored as ll_exact) is reproduced
    here, it does not depend on its own blocking beyond a small fraction of
    the FP64 error scale, and where K is well conditioned it agrees with the
    FP64 oracle to ~1e-13."""
    c = load_case(name)
    ks = [int(v) for v in c["kspec"]]
    for k, th in enumerate(c["thetas"][:2]):
        args = (ks, th, c["X"], c["y"], c["mu"], int(c["likelihood"]), float(c["noise"]), bool(c["optimise_noise"]))
        a = E.loglik_ld(*args)[0]
        b = E.loglik_ld(*args, nb=40)[0]
        ex, err = float(c["ll_exact"][k]), float(c["fp64_err"][k])
        assert abs(a - ex) <= 1e-14 * abs(ex)
        assert abs(a - b) <= max(0.01 * err, 4e-16 * abs(ex)), (a, b, err)
        if err <= 1e-12 * abs(ex):
            assert abs(ex - c["ll"][k]) <= 1e-12 * abs(ex)


def test_extended_precision_kernel_matches_the_fp64_kernel():
    rng = np.random.default_rng(5)
    X = rng.normal(2.0, 0.2, size=(50, 5))
    X[:, 4] = rng.uniform(-3.0, 3.0, size=50)
    ks = [O.RBF, 4, 1, 2, 3, 4, O.PERIODIC, 1, 5, O.PROD, O.CONSTANT, 0, O.SUM]
    th = rng.uniform(0.0, 1.0, size=O.kernel_nparams(ks))
    K = O.compute_R(ks, th, 1e-8, O.Tensors(X))
    Kl = E.compute_R_ld(ks, th, 1e-8, X).astype(np.float64)
    low = np.tril(np.ones_like(K)).astype(bool)
    assert np.max(np.abs(K - Kl)[low]) <= 8e-16 * np.max(np.abs(K))


def _data(n=40, d=4, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(0.0, 1.0, size=(n, d))
    y = np.sin(X[:, 0]) + 0.1 * rng.normal(size=n)
    return X, y


def test_rbf_tensor_path_matches_pairwise_k():
    X, _ = _data()
    ls = np.array([1.3, 0.7, 2.0])
    dims = [0, 2, 3]
    R = O.leaf_R(O.RBF, dims, ls, O.Tensors(X))
    for i in range(0, 40, 7):
        for j in range(0, i + 1, 5):
            k = O.pairwise_k(O.RBF, dims, ls, X[i], X[j])
            assert abs(R[i, j] - k) <= 4e-15 * abs(k)


def test_periodic_tensor_path_matches_half_angle_formula():
    X, _ = _data()
    ls = np.array([0.4, 0.9])
    dims = [1, 3]
    R = O.leaf_R(O.PERIODIC, dims, ls, O.Tensors(X))
    for i in range(0, 40, 3):
        for j in range(0, i + 1, 4):
            s = sum(l * math.sin(abs(X[i, d] - X[j, d]) / 2.0) ** 2 for l, d in zip(ls, dims))
            assert abs(R[i, j] - math.exp(-2.0 * s)) <= 4e-15


def test_lazy_and_tensor_modes_agree():
    X, y = _data(60, 5, 3)
    ks = [O.RBF, 3, 1, 2, 4, O.PERIODIC, 2, 3, 5, O.PROD]
    th = np.array([0.2, 0.5, 0.1, 0.3, 0.7])
    mu = O.mean_vector("constant", X, y)
    a, _ = O.loglik(ks, th, X, y, mu, 0, 1e-6, False, tens=O.Tensors(X, lazy=False))
    b, _ = O.loglik(ks, th, X, y, mu, 0, 1e-6, False, tens=O.Tensors(X, lazy=True))
    assert abs(a - b) <= 1e-11 * abs(a)


def test_lapack_cholesky_matches_python_cholesky():
    X, _ = _data(50, 3, 1)
    K = O.compute_R([O.RBF, 3, 1, 2, 3], np.zeros(3), 1e-3, O.Tensors(X))
    L1, i1 = O.cholesky(K)
    L2, i2 = O.cholesky_python(np.tril(K) + np.tril(K, -1).T)
    assert i1 == i2 == 0
    assert abs(O.log_determinant(L1) - O.log_determinant(L2)) <= 1e-11 * abs(O.log_determinant(L1))
    assert np.max(np.abs(np.tril(L1) - L2)) <= 1e-12


def test_lapack_cholesky_matches_torch_mkl():
    torch = pytest.importorskip("torch")
    X, _ = _data(80, 4, 2)
    K = O.compute_R([O.RBF, 4, 1, 2, 3, 4], np.full(4, -1.0), 1e-4, O.Tensors(X))
    L1, _ = O.cholesky(K)
    L2 = torch.linalg.cholesky(torch.tensor(np.tril(K) + np.tril(K, -1).T)).numpy()
    assert np.max(np.abs(np.tril(L1) - L2)) <= 1e-10


def test_not_positive_definite_reports_lapack_info():
    X, y = _data(30, 2, 4)
    X = np.vstack([X, X[:5]])
    y = np.concatenate([y, y[:5]])
    ll, info = O.loglik([O.RBF, 2, 1, 2], np.array([1.0, 1.0]), X, y, O.mean_vector("zero", X, y), 0, 0.0,
                        False)
    assert info == 31 and math.isnan(ll)  # first duplicated row


def test_concentrated_mean_is_the_gls_optimum():
    X, y = _data(45, 3, 5)
    ks = [O.RBF, 3, 1, 2, 3]
    th = np.array([0.3, 0.1, 0.5])
    r = O.loglik(ks, th, X, y, None, 1, 1e-6, False, want=True)
    K = O.compute_R(ks, th, 1e-6, O.Tensors(X))
    K = np.tril(K) + np.tril(K, -1).T
    def q(m):
        v = y - m
        return v @ np.linalg.solve(K, v)
    m = r["mean"]
    assert q(m) <= q(m + 1e-4) and q(m) <= q(m - 1e-4)
    assert abs(r["sigma2"] - q(m) / len(y)) <= 1e-9 * r["sigma2"]


@pytest.mark.parametrize("lik", [0, 1])
def test_analytic_gradient_matches_central_differences(lik):
    X, y = _data(35, 3, 6)
    ks = [O.RBF, 2, 1, 2, O.PERIODIC, 1, 3, O.PROD]
    th = np.array([0.4, 0.2, 0.6, 3e-3])
    mu = O.mean_vector("constant", X, y)
    ll, g, info = O.loglik_grad(ks, th, X, y, mu, lik, 1e-6, True)
    fd = O.central_fd(ks, th, X, y, mu, lik, 1e-6, True, rel=1e-5)
    assert info == 0
    assert np.allclose(g, fd, rtol=1e-5, atol=1e-6 * np.max(np.abs(fd)))


def test_mean_functions_host_mirror_matches_oracle():
    from fgpu.gpr import mean_vector
    X, y = _data(60, 4, 7)
    for kind in ("zero", "constant", "linear", "quadratic"):
        a = mean_vector(kind, X, y)
        b = O.mean_vector(kind, X, y)
        assert np.allclose(a, b, rtol=1e-10, atol=1e-12), kind


@pytest.mark.parametrize("lik", [0, 1])
def test_columnwise_gradient_matches_dense(lik):
    X, y = _data(50, 4, 11)
    ks = [O.RBF, 2, 1, 2, O.PERIODIC, 1, 4, O.PROD, O.CONSTANT, 0, O.SUM, O.LINEAR, 1, 3, O.SUM]
    th = np.array([0.3, 0.5, 0.2, 0.7, 0.1, 2e-4])
    mu = O.mean_vector("constant", X, y)
    _, a, _ = O.loglik_grad(ks, th, X, y, mu, lik, 1e-5, True)
    _, b, _ = O.loglik_grad_columns(ks, th, X, y, mu, lik, 1e-5, True)
    assert np.allclose(a, b, rtol=1e-9, atol=1e-12)
