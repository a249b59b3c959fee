"""The adjoint (fgpu_grad) against the oracle's analytic FP64 gradient and
central finite differences.

Target: d logL / d theta within 1e-6 relative of the FP64 oracle.  Per
component: |g - g_ref| <= 1e-6 |g_ref| + 1e-9 max|g_ref| (the absolute slack
covers components that cancel to ~0).
"""
import numpy as np
import pytest

from oracle import gpr_oracle as O

pytestmark = pytest.mark.gpu


def _problem(n, d, seed, per=True):
    rng = np.random.default_rng(seed)
    X = rng.normal(2.0, 0.3, size=(n, d))
    X[:, -1] = rng.uniform(-np.pi, np.pi, size=n)
    y = np.cos(X[:, 0]) + 0.3 * np.sin(X[:, -1]) + 0.05 * X[:, 1] + 1e-3 * rng.normal(size=n)
    return X, y


KERNELS = {
    "rbf_plus_per": lambda d: [O.RBF, d - 1] + list(range(1, d)) + [O.PERIODIC, 1, d, O.SUM],
    "rbf_times_per": lambda d: [O.RBF, d - 1] + list(range(1, d)) + [O.PERIODIC, 1, d, O.PROD],
    "prod_plus_const": lambda d: [O.RBF, 2, 1, 2, O.PERIODIC, 1, d, O.PROD, O.CONSTANT, 0, O.SUM],
    "linear_in_sum": lambda d: [O.RBF, d, *range(1, d + 1), O.LINEAR, 1, 2, O.SUM],
    "cyclic": lambda d: [O.RBF_CYCLIC, d, *range(1, d + 1)],
}


def close(g, ref, rel=1e-6):
    g, ref = np.asarray(g), np.asarray(ref)
    return np.all(np.abs(g - ref) <= rel * np.abs(ref) + 1e-9 * np.max(np.abs(ref)) + 1e-30)


@pytest.mark.parametrize("kern", sorted(KERNELS))
@pytest.mark.parametrize("lik", [0, 1])
@pytest.mark.parametrize("noise_opt", [False, True])
def test_grad_matches_oracle(kern, lik, noise_opt, lib):
    from fgpu import Engine
    n, d = 150, 4
    X, y = _problem(n, d, seed=hash((kern, lik, noise_opt)) % 1000)
    ks = KERNELS[kern](d)
    mu = O.mean_vector("constant", X, y)
    nk = O.kernel_nparams(ks)
    rng = np.random.default_rng(7)
    th = rng.uniform(0.05, 0.9, size=nk + (1 if noise_opt else 0))
    if noise_opt:
        th[nk] = 1e-4
    noise = 1e-5
    e = Engine(X, y, mu, ks, lik, noise, noise_opt)
    ll, g, info = e.grad(th)
    rll, rg, rinfo = O.loglik_grad(ks, th, X, y, mu, lik, noise, noise_opt)
    assert info == rinfo == 0
    assert abs(ll - rll) <= 1e-9 * abs(rll)
    assert close(g, rg), (g, rg)
    # the plain path gives the same likelihood
    l2, i2 = e.loglik(th)
    assert i2 == 0 and abs(l2 - ll) <= 1e-9 * abs(ll)


@pytest.mark.parametrize("n", [1, 63, 64, 65, 130])
def test_grad_edge_sizes(n, lib):
    from fgpu import Engine
    X, y = _problem(n, 3, seed=n)
    ks = KERNELS["rbf_plus_per"](3)
    mu = O.mean_vector("constant", X, y)
    th = np.array([0.3, 0.6, 0.2])
    e = Engine(X, y, mu, ks, 0, 1e-4, False)
    ll, g, info = e.grad(th)
    rll, rg, rinfo = O.loglik_grad(ks, th, X, y, mu, 0, 1e-4, False)
    assert info == rinfo == 0
    assert abs(ll - rll) <= 1e-9 * abs(rll)
    assert close(g, rg)


def test_grad_glycine_like_against_oracle_and_fd(lib, fp64_trailing):
    """The glycine-like configuration's kernel (rbf over 17 dims + periodic over
    7 dihedrals, concentrated likelihood, 24 parameters) at N=600 against the
    oracle, and the adjoint against central differences of the engine's own
    log-likelihood (h = 1e-6 theta, the benchmark configuration's step) on the
    FP64 trailing update: the tensor-core path's rounding differs between
    nearby theta by ~1e-13 |logL| (its smoothness is tested at full size
    below with a step fitted to that), which a 2-point difference with this
    step turns into ~1e-13 |logL| / h, the size of the allowance itself."""
    from fgpu import Engine, loglik_batch, synth
    p = synth.config3(600)
    mu = O.mean_vector("constant", p.X, p.y)
    e = Engine(p.X, p.y, mu, p.kspec, p.likelihood, p.noise, False)
    th = p.thetas(1, seed=3)[0]
    ll, g, info = e.grad(th)
    rll, rg, rinfo = O.loglik_grad(p.kspec, th, p.X, p.y, mu, p.likelihood, p.noise, False)
    assert info == rinfo == 0
    assert close(g, rg), np.max(np.abs(g - rg) / np.maximum(np.abs(rg), 1e-300))
    plus, minus = [], []
    for q in range(len(th)):
        h = 1e-6 * th[q]
        tp, tm = th.copy(), th.copy()
        tp[q] += h
        tm[q] -= h
        plus.append(tp)
        minus.append(tm)
    lp, ip = loglik_batch([e] * len(th), plus)
    lm, im = loglik_batch([e] * len(th), minus)
    den = np.array([tp[q] - tm[q] for q, (tp, tm) in enumerate(zip(plus, minus))])
    fd = (lp - lm) / den
    assert np.all(ip == 0) and np.all(im == 0)
    # central differences carry the log-likelihood's own rounding divided by
    # the step: allow 1e-5 relative plus 1e-13 |ll| / h
    tol = 1e-5 * np.abs(fd) + 1e-13 * abs(ll) / (0.5 * den)
    assert np.all(np.abs(g - fd) <= tol), (g - fd, tol)


def test_grad_not_positive_definite_reports_info(lib):
    from fgpu import Engine
    X, y = _problem(40, 3, seed=5)
    X = np.vstack([X, X[:10]])
    y = np.concatenate([y, y[:10]])
    ks = [O.RBF, 3, 1, 2, 3]
    e = Engine(X, y, O.mean_vector("zero", X, y), ks, 0, 0.0, False)
    ll, g, info = e.grad(np.array([1.0, 1.0, 1.0]))
    assert info > 0 and np.isnan(ll) and np.all(np.isnan(g))


@pytest.fixture
def fp64_trailing():
    from fgpu.gpr import set_trailing_update
    prev = set_trailing_update("fp64")
    yield
    set_trailing_update(prev)


def _stencil(engine, th, hs):
    """5-point central differences of the engine's log-likelihood."""
    from fgpu import loglik_batch
    pts = []
    for q in range(len(th)):
        for m in (2, 1, -1, -2):
            t = th.copy()
            t[q] += m * hs[q]
            pts.append(t)
    lv, iv = loglik_batch([engine] * len(pts), pts)
    assert np.all(iv == 0)
    lv = lv.reshape(len(th), 4)
    return (-lv[:, 0] + 8 * lv[:, 1] - 8 * lv[:, 2] + lv[:, 3]) / (12 * np.asarray(hs))


@pytest.mark.parametrize("seed", [5, 8])
def test_grad_full_size_glycine_like_against_fd(seed, lib, fp64_trailing):
    """N=4000, d=24, 24 parameters (the benchmark workload): the adjoint
    against a 5-point central-difference stencil of the log-likelihood with
    the FP64 trailing update.  At this size logL carries ~1e-10 of rounding
    jitter, so a step of 1e-6 theta would leave 1e-4 of noise in a 2-point
    difference; h = 1e-4 theta with the O(h^4) stencil keeps both truncation
    and noise well below 1e-5 relative (measured: at most 1.6e-6)."""
    from fgpu import Engine, synth
    p = synth.config3()
    mu = O.mean_vector("constant", p.X, p.y)
    e = Engine(p.X, p.y, mu, p.kspec, p.likelihood, p.noise, False)
    th = p.thetas(1, seed=seed)[0]
    ll, g, info = e.grad(th)
    assert info == 0
    l2, i2 = e.loglik(th)
    assert i2 == 0 and abs(l2 - ll) <= 1e-9 * abs(ll)
    fd = _stencil(e, th, 1e-4 * th)
    rel_fd = np.max(np.abs(g - fd) / np.abs(fd))
    assert rel_fd <= 1e-5, rel_fd
    if seed != 5:
        return
    # the FP64 oracle gradient at full size (column-wise, same formula)
    rll, rg, rinfo = O.loglik_grad_columns(p.kspec, th, p.X, p.y, mu, p.likelihood, p.noise, False)
    assert rinfo == 0 and abs(ll - rll) <= 1e-9 * abs(rll)
    assert close(g, rg), np.max(np.abs(g - rg) / np.abs(rg))


@pytest.mark.parametrize("seed", [5, 8])
def test_tensor_core_loglik_smooth_at_full_size(seed, lib):
    """The same stencil on the tensor-core path's log-likelihood.  Its value
    sits within ~1e-11 relative of the FP64 path, but its rounding differs
    between nearby theta by ~1e-13 |logL| (55-bit fixed-point digits with
    their scale per row, fresh for every evaluation), which the stencil
    divides by h = 1e-4 theta: up to ~2e-5 relative on the smallest
    components (measured on four theta), so the bound here is 1e-4.  The
    likelihood itself is checked against the oracle to 1e-9 elsewhere."""
    from fgpu import Engine, synth
    p = synth.config3()
    mu = O.mean_vector("constant", p.X, p.y)
    e = Engine(p.X, p.y, mu, p.kspec, p.likelihood, p.noise, False)
    th = p.thetas(1, seed=seed)[0]
    ll, g, info = e.grad(th)
    assert info == 0
    fd = _stencil(e, th, 1e-4 * th)
    rel_fd = np.abs(g - fd) / np.abs(fd)
    assert np.max(rel_fd) <= 1e-4, np.max(rel_fd)
    assert np.median(rel_fd) <= 1e-6, np.median(rel_fd)
