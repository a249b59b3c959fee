"""Extended-precision log-likelihood: the "exact" value FP64 codes are measured against.

TEST INFRASTRUCTURE ONLY (like the rest of ``oracle/``): nothing in the
product imports it; the tests and the fixture generator use it as a checker.

Why it exists.  With the reference's default nugget of 1e-10
(src/config/model_config.f90:42-54) the kernel matrix of a smooth data set
is nearly singular (cond(K) ~ 1e10-1e12), and two standard FP64 LAPACKs
evaluating the same formulas on the same K disagree by up to ~1e-5 of logL
(OpenBLAS vs MKL on the water-like set).  Neither is "the" answer, so an FP64
code cannot be measured by its distance to one of them.  This module evaluates
the reference's formulas with a 64-bit significand instead of 53 bits
(numpy ``longdouble``: x87 80-bit extended on x86-64, IEEE binary128 on
aarch64), so its result is ~2000 times (x86-64) or more closer to the exact
logL of the FP64 inputs than any FP64 evaluation; FP64 codes are then
measured by their distance to it.

What it restates (paths in the FEREBUS-v7 source tree), with every
intermediate in extended precision:

* parameter transforms   src/kernels/rbf_kernel.f90:113-119 (l = exp(theta)),
                         src/kernels/periodic_kernel.f90:111-118 (l = exp(-theta)^2),
                         src/kernels/linear_kernel.f90:94-100, src/kernels/constant.f90:86-90
* kernel values          rbf exp(-1/2 sum_k l_k (x_ik - x_jk)^2) (stationary_kernel.f90:101-122),
                         periodic exp(-2 sum_k l_k sin^2(|x_ik - x_jk| / 2)) (periodic_kernel.f90:181-206),
                         rbf-cyclic with every 3rd feature wrapped (distance_matrix.f90:95-128),
                         linear (order 0) and constant (kernel_module.f90:208-219)
* sum / product, nugget  kernel_module.f90:309-375, gpr.f90:185-189
* Cholesky, log-det      likelihood.f90:130-159, arith.f90:72-93 (2 sum log L_ii)
* marginal / concentrated likelihood.f90:161-253

The Cholesky is a blocked right-looking factorisation written here (numpy
has no extended-precision LAPACK); trailing updates are extended-precision
matrix products.  ``loglik_ld`` returns the value rounded to a double.
"""
from __future__ import annotations

import numpy as np

from . import gpr_oracle as O

LD = np.longdouble
PI_LD = LD("3.14159265358979323846264338327950288")
TWOPI_LD = 2 * PI_LD
LOG_TWOPI_LD = np.log(TWOPI_LD)


def _leaf_params_ld(op, theta):
    t = np.asarray(theta, dtype=np.float64).astype(LD)
    if op in (O.RBF, O.RBF_CYCLIC):
        return np.exp(t)
    if op == O.PERIODIC:
        ls = LD(1) / np.exp(t)
        return ls * ls
    if op == O.LINEAR:
        return np.exp(-t)
    if op == O.CONSTANT:
        return t.copy()
    raise ValueError(op)


def _wrap_ld(c):
    """distance_matrix.f90:119-120: sign(c) * (mod(|c| + pi, 2 pi) - pi)."""
    a = np.abs(c) + PI_LD
    w = (a - np.trunc(a / TWOPI_LD) * TWOPI_LD) - PI_LD
    return np.where(c == 0, LD(0), np.where(c < 0, -w, w))


def kernel_R_ld(kspec, theta, X, rows=None):
    """k(X, X) in extended precision (dense, symmetric).  ``rows``: optional
    subset of row indices (all columns) to bound memory."""
    X = np.asarray(X, dtype=np.float64).astype(LD)
    n, d = X.shape
    ri = np.arange(n) if rows is None else np.asarray(rows)
    diff = X[ri][:, None, :] - X[None, :, :]          # (m, n, d)
    stack, p = [], 0
    for node in O.parse_kspec(kspec):
        if node[0] == "leaf":
            _, op, dims = node
            k = O.leaf_nparams(op, dims)
            prm = _leaf_params_ld(op, np.asarray(theta, dtype=np.float64)[p:p + k])
            p += k
            if op == O.RBF:
                v = np.exp(LD(-0.5) * np.einsum("mnk,k->mn", diff[:, :, dims] ** 2, prm))
            elif op == O.PERIODIC:
                s = np.sin(np.abs(diff[:, :, dims]) / 2)
                v = np.exp(LD(-2) * np.einsum("mnk,k->mn", s * s, prm))
            elif op == O.RBF_CYCLIC:
                dc = diff.copy()
                cyc = np.arange(2, d, 3)
                dc[:, :, cyc] = _wrap_ld(dc[:, :, cyc])
                v = np.exp(LD(-0.5) * np.einsum("mnk,k->mn", dc ** 2, prm))
            elif op == O.LINEAR:
                v = np.full((len(ri), n), np.sum(LD(1) / prm), dtype=LD)
            else:
                v = np.full((len(ri), n), prm[0], dtype=LD)
            stack.append(v)
        else:
            b = stack.pop()
            a = stack.pop()
            stack.append(a + b if node[1] == O.SUM else a * b)
    return stack[0]


def compute_R_ld(kspec, theta, noise, X, chunk=None):
    """K = k(X, X) + noise I in extended precision, built in row chunks
    (about 2e7 pairwise differences per chunk)."""
    n, d = np.asarray(X).shape
    if chunk is None:
        chunk = max(1, int(2e7 // (n * d)))
    K = np.empty((n, n), dtype=LD)
    for r0 in range(0, n, chunk):
        rows = np.arange(r0, min(n, r0 + chunk))
        K[rows] = kernel_R_ld(kspec, theta, X, rows)
    K[np.arange(n), np.arange(n)] += LD(float(noise))
    return K


def cholesky_ld(K, nb=64):
    """Blocked right-looking Cholesky (lower) in place on a copy; returns
    (L, info) with info the 1-based column of the first non-positive pivot,
    as dpotrf reports it."""
    A = np.array(K, dtype=LD)
    n = A.shape[0]
    for k0 in range(0, n, nb):
        k1 = min(n, k0 + nb)
        for j in range(k0, k1):
            if not A[j, j] > 0:
                return A, j + 1
            A[j, j] = np.sqrt(A[j, j])
            A[j + 1:k1, j] /= A[j, j]
            c = A[j + 1:k1, j]
            A[j + 1:k1, j + 1:k1] -= np.outer(c, c)
        if k1 < n:
            # panel: rows below the block solve x L11^T = a (forward substitution)
            P = A[k1:, k0:k1]
            for j in range(k1 - k0):
                if j:
                    P[:, j] -= P[:, :j] @ A[k0 + j, k0:k0 + j]
                P[:, j] /= A[k0 + j, k0 + j]
            A[k1:, k0:k1] = P
            # trailing update, lower block columns only
            for c0 in range(k1, n, nb):
                c1 = min(n, c0 + nb)
                A[c0:, c0:c1] -= P[c0 - k1:] @ P[c0 - k1:c1 - k1].T
    return np.tril(A), 0


def _solve_ld(L, b):
    """x = (L L^T)^-1 b by forward and back substitution (dpotrs)."""
    n = L.shape[0]
    z = np.array(b, dtype=LD)
    for i in range(n):
        z[i] = (z[i] - L[i, :i] @ z[:i]) / L[i, i]
    x = z
    for i in range(n - 1, -1, -1):
        x[i] = (x[i] - L[i + 1:, i] @ x[i + 1:]) / L[i, i]
    return x


def loglik_ld(kspec, theta, X, y, mu, likelihood, noise, optimise_noise, nb=64, want=False):
    """The reference's log-likelihood (gpr.f90:258-307, likelihood.f90:130-253)
    in extended precision.  Returns (ll, info) with ll rounded to a double."""
    theta = np.asarray(theta, dtype=np.float64)
    nk = O.kernel_nparams(kspec)
    if optimise_noise:
        noise = float(theta[nk])
    K = compute_R_ld(kspec, theta[:nk], noise, X)
    L, info = cholesky_ld(K, nb=nb)
    if info:
        return (float("nan"), info) if not want else {"ll": float("nan"), "info": info}
    n = L.shape[0]
    logdet = 2 * np.sum(np.log(np.diag(L)))
    y = np.asarray(y, dtype=np.float64).astype(LD)
    if likelihood == O.MARGINAL:
        r = y - np.asarray(mu, dtype=np.float64).astype(LD)
        a = _solve_ld(L, r)
        ll = LD(-0.5) * (r @ a) - logdet / 2 - LD(n) * LOG_TWOPI_LD / 2
    else:
        ry = _solve_ld(L, y)
        r1 = _solve_ld(L, np.ones(n, dtype=LD))
        m = np.sum(ry) / np.sum(r1)
        r = y - m
        a = _solve_ld(L, r)
        s2 = (r @ a) / n
        ll = LD(-0.5) * n * np.log(s2) - logdet / 2
    if want:
        return {"ll": float(ll), "info": 0, "ll_ld": ll, "logdet": float(logdet)}
    return float(ll), 0


def fp64_error_scale(kspec, theta, X, y, mu, likelihood, noise, optimise_noise, ll_exact, trials=8, seed=0):
    """The FP64 error scale of one likelihood, computed on the spot: the
    largest |ll' - ll_exact| over the FP64 oracle (OpenBLAS) and the oracle
    on `trials` random symmetric 4-ulp perturbations of K.  Returns
    (scale, OpenBLAS value)."""
    theta = np.asarray(theta, dtype=np.float64)
    nk = O.kernel_nparams(kspec)
    if optimise_noise:
        noise = float(theta[nk])
    tens = O.Tensors(X, need_cyclic=O.RBF_CYCLIC in list(kspec))
    K = O.compute_R(kspec, theta[:nk], noise, tens)
    K = np.tril(K) + np.tril(K, -1).T
    y = np.asarray(y, dtype=np.float64)
    mu = np.asarray(mu, dtype=np.float64)
    n = K.shape[0]

    def ll_of(Km):
        L, info = O.cholesky(Km)
        if info:
            return float("nan")
        logdet = O.log_determinant(L)
        if likelihood == O.MARGINAL:
            r = y - mu
            return -0.5 * float(r @ O.potrs(L, r)) - 0.5 * logdet - 0.5 * n * O.LOG_TWOPI
        ry, r1 = O.potrs(L, y), O.potrs(L, np.ones(n))
        m = float(ry.sum()) / float(r1.sum())
        r = y - m
        return -0.5 * n * np.log(float(r @ O.potrs(L, r)) / n) - 0.5 * logdet

    ob = ll_of(K)
    worst = abs(ob - ll_exact)
    rng = np.random.default_rng(seed)
    u = np.finfo(np.float64).eps / 2
    for _ in range(trials):
        P = rng.uniform(-4 * u, 4 * u, size=K.shape)
        P = np.tril(P) + np.tril(P, -1).T
        v = ll_of(K * (1.0 + P))
        if np.isfinite(v):
            worst = max(worst, abs(v - ll_exact))
    return worst, ob
