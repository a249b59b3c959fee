"""CPU oracle for the GPR log-likelihood hot path of FEREBUS-v7.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may use it, and only as the checker
(or the timed CPU baseline), never as the thing measured on the GPU.

What it restates (all paths relative to the FEREBUS-v7 source tree):

* kernel parameter transforms      src/kernels/rbf_kernel.f90:113-119,
                                   src/kernels/periodic_kernel.f90:111-118,
                                   src/kernels/rbf_cyclic_kernel.f90:109-115,
                                   src/kernels/linear_kernel.f90:94-100,
                                   src/kernels/constant.f90:86-90
* composite parameter split        src/kernels/kernel_module.f90:235-245
* distance tensors                 src/kernels/distance_matrix.f90:64-142
* R for rbf / periodic (CPU path)  src/kernels/stationary_kernel.f90:101-122,
                                   src/kernels/periodic_kernel.f90:181-206
* R for rbf-cyclic                 src/kernels/stationary_cyclic_kernel.f90:104-127
* R for linear / constant          src/kernels/kernel_module.f90:208-219 (pairwise loop)
* sum / product                    src/kernels/kernel_module.f90:309-325, 359-375
* nugget                           src/model/gpr/gpr.f90:185-189
* Cholesky + log-det               src/model/gpr/likelihood.f90:130-159,
                                   src/utils/arith.f90:72-93, src/utils/linalg.f90:73-98
* marginal / concentrated logL     src/model/gpr/likelihood.f90:161-253
* mean functions                   src/mean/constant.f90:42-55, src/mean/least_squares.f90:54-93,
                                   src/mean/linear.f90:41-51, src/mean/quadratic.f90:41-52,
                                   src/mean/zero.f90:47-52

LAPACK: the reference calls ``dpotrf('L')`` / ``dpotrs('L')`` / ``dposv('L')``
from OpenBLAS (or netlib lapack-3.8.0); here the same routines come from
scipy's bundled OpenBLAS through ``scipy.linalg.lapack``.

PARITY UNPINNED: the reference ships no tests, golden vectors or known-answer
tests, and it cannot be built in this environment (pure Fortran, no Fortran
compiler, its toml-f dependency is an empty submodule).  This restatement is
cross-checked only against restatements: the distance-tensor path against
the pairwise ``k`` path of the same kernels, OpenBLAS against an independent
LAPACK (torch/MKL) and a pure-Python Cholesky, the analytic gradient against
central finite differences, the C restatement (ref_cpu.c) against this
module's fixtures, and the extended-precision evaluation (exact.py) that
parity is measured against, against 40-digit mpmath arithmetic.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.linalg import lapack

# Kernel-spec opcodes.  The spec is the postfix flattening of the kernel
# expression tree: a leaf is ``[op, n_active, dim_1, ..., dim_n]`` (1-based
# feature indices, as in the TOML ``active_dimensions``), an operator is
# ``[op]``.  The same encoding crosses the C-ABI.
RBF, PERIODIC, RBF_CYCLIC, LINEAR, CONSTANT = 1, 2, 3, 4, 5
SUM, PROD = 10, 11
LEAF_OPS = (RBF, PERIODIC, RBF_CYCLIC, LINEAR, CONSTANT)

MARGINAL, CONCENTRATED = 0, 1

PI = 4.0 * math.atan(1.0)          # src/constants.f90:30
TWOPI = 2.0 * PI                   # src/constants.f90:31
LOG_TWOPI = math.log(TWOPI)        # src/constants.f90:32


# --------------------------------------------------------------------------
# kernel spec
# --------------------------------------------------------------------------
def parse_kspec(kspec):
    """Split a postfix kernel spec into a list of nodes.

    Each node is ``("leaf", op, dims0)`` with 0-based dims, or ``("op", op)``.
    """
    nodes, i, ks = [], 0, list(kspec)
    while i < len(ks):
        op = ks[i]
        if op in LEAF_OPS:
            n = ks[i + 1]
            dims = [d - 1 for d in ks[i + 2:i + 2 + n]]
            nodes.append(("leaf", op, dims))
            i += 2 + n
        elif op in (SUM, PROD):
            nodes.append(("op", op))
            i += 1
        else:
            raise ValueError(f"bad kernel-spec opcode {op} at {i}")
    return nodes


def leaf_nparams(op, dims):
    """Number of hyperparameters of one leaf kernel."""
    return 1 if op == CONSTANT else len(dims)


def kernel_nparams(kspec):
    """Number of kernel hyperparameters (``Kernel%nparams``)."""
    return sum(leaf_nparams(n[1], n[2]) for n in parse_kspec(kspec) if n[0] == "leaf")


def leaf_transform(op, theta):
    """Raw parameters -> the stored kernel parameters.

    rbf / rbf-cyclic: lengthscale = exp(theta)           (rbf_kernel.f90:113-119)
    periodic:         lengthscale = (1/exp(theta))**2     (periodic_kernel.f90:111-118)
    linear:           c = exp(-theta)                     (linear_kernel.f90:94-100)
    constant:         value = theta                       (constant.f90:86-90)
    """
    theta = np.asarray(theta, dtype=np.float64)
    if op in (RBF, RBF_CYCLIC):
        return np.exp(theta)
    if op == PERIODIC:
        ls = 1.0 / np.exp(theta)
        return ls * ls
    if op == LINEAR:
        return np.exp(-theta)
    if op == CONSTANT:
        return theta.copy()
    raise ValueError(op)


# --------------------------------------------------------------------------
# distance tensors (distance_matrix.f90)
# --------------------------------------------------------------------------
def distance_tensor(X):
    """D(f, i, j) = (x_if - x_jf)**2 for i > j, 0 on the diagonal.

    distance_matrix.f90:64-93.  The strict upper triangle is never written by
    the reference; it is left at zero here and never read.
    """
    X = np.asarray(X, dtype=np.float64)
    n, d = X.shape
    D = np.zeros((d, n, n))
    xt = X.T
    for j in range(n):
        diff = xt[:, j + 1:] - xt[:, j:j + 1]
        D[:, j + 1:, j] = diff * diff
    return D


def cyclic_distance_tensor(X):
    """As ``distance_tensor`` but every 3rd feature (3, 6, 9, ... 1-based) is
    wrapped to [-pi, pi] before squaring: distance_matrix.f90:95-128."""
    X = np.asarray(X, dtype=np.float64)
    n, d = X.shape
    D = np.zeros((d, n, n))
    xt = X.T
    cyc = np.arange(2, d, 3)
    for j in range(n):
        diff = xt[:, j + 1:] - xt[:, j:j + 1]
        c = diff[cyc]
        # Fortran mod(a, p) = a - int(a/p)*p; a = |c| + pi > 0 here.
        a = np.abs(c) + PI
        diff[cyc] = np.sign(c) * ((a - np.trunc(a / TWOPI) * TWOPI) - PI)
        # Fortran sign(1.0, 0.0) = +1
        zero = c == 0.0
        if zero.any():
            diff[cyc] = np.where(zero, (a - np.trunc(a / TWOPI) * TWOPI) - PI, diff[cyc])
        D[:, j + 1:, j] = diff * diff
    return D


def periodic_tensor(D):
    """P = sin(sqrt(D)/2)**2 over the whole tensor: distance_matrix.f90:130-142."""
    P = np.sin(np.sqrt(D) / 2.0)
    return P * P


class Tensors:
    """The per-data-set tensors the reference precomputes (app/main.f90:108).

    With ``lazy=True`` (large N) the d x N x N tensors are not stored: each
    column j of D / P is formed when R's column j is evaluated, with the same
    arithmetic (diff*diff, sin(sqrt(D)/2)**2, alpha * D^T l, exp).
    """

    def __init__(self, X, need_cyclic=False, lazy=None):
        self.X = np.asarray(X, dtype=np.float64)
        n, d = self.X.shape
        self.lazy = (n * n * d > 60_000_000) if lazy is None else bool(lazy)
        if self.lazy:
            self.D = self.P = self.C = None
            return
        self.D = distance_tensor(self.X)
        self.P = periodic_tensor(self.D)
        self.C = cyclic_distance_tensor(self.X) if need_cyclic else None

    def column(self, j):
        """D(:, j:, j), P(:, j:, j) and the cyclic D(:, j:, j) for column j."""
        xt = self.X.T
        diff = xt[:, j:] - xt[:, j:j + 1]
        D = diff * diff
        P = np.sin(np.sqrt(D) / 2.0)
        P = P * P
        cyc = np.arange(2, xt.shape[0], 3)
        dc = diff.copy()
        c = dc[cyc]
        a = np.abs(c) + PI
        dc[cyc] = np.where(c == 0.0, 0.0, np.sign(c) * ((a - np.trunc(a / TWOPI) * TWOPI) - PI))
        return D, P, dc * dc


# --------------------------------------------------------------------------
# kernel matrix R (lower triangle + diagonal meaningful)
# --------------------------------------------------------------------------
def _gemv_t(T, dims, w, alpha):
    """R = alpha * T(dims,:,:)^T w  -- the dgemv('t') of stationary_kernel.f90:110-119."""
    n = T.shape[1]
    sel = T[dims].reshape(len(dims), n * n)
    return (alpha * (w @ sel)).reshape(n, n)


def leaf_R(op, dims, params, tens: Tensors):
    X = tens.X
    n, d = X.shape
    if tens.lazy and op in (RBF, PERIODIC, RBF_CYCLIC):
        if op == RBF_CYCLIC and len(dims) != d:
            raise ValueError("rbf-cyclic requires active_dims == all features (reference shape rule)")
        # blocks of columns j0..j1-1, rows j0..n-1, with the same arithmetic as
        # the stored tensors: diff*diff, sin(sqrt(D)/2)**2, l . D over the
        # dims (a dgemv in the reference), exp
        R = np.zeros((n, n))
        B = max(1, int(4e6 // (n * max(len(dims), 1))))
        for j0 in range(0, n, B):
            j1 = min(n, j0 + B)
            diff = X[j0:, None, dims] - X[None, j0:j1, dims]        # (n - j0, b, k)
            if op == RBF_CYCLIC:
                cyc = [q for q, dm in enumerate(dims) if dm % 3 == 2]
                c = diff[:, :, cyc]
                a = np.abs(c) + PI
                diff[:, :, cyc] = np.where(c == 0.0, 0.0, np.sign(c) * ((a - np.trunc(a / TWOPI) * TWOPI) - PI))
            D = diff * diff
            if op == PERIODIC:
                P = np.sin(np.sqrt(D) / 2.0)
                R[j0:, j0:j1] = np.exp(-2.0 * ((P * P) @ params))
            else:
                R[j0:, j0:j1] = np.exp(-0.5 * (D @ params))
        return R
    if op == RBF:
        return np.exp(_gemv_t(tens.D, dims, params, -0.5))
    if op == PERIODIC:
        return np.exp(_gemv_t(tens.P, dims, params, -2.0))
    if op == RBF_CYCLIC:
        # stationary_cyclic_kernel.f90:104-127: the lengthscale vector is
        # applied to the cyclic tensor over *all* features.
        if len(dims) != d:
            raise ValueError("rbf-cyclic requires active_dims == all features (reference shape rule)")
        s = np.tensordot(params, tens.C, axes=1)
        return np.exp(-0.5 * s)
    if op == LINEAR:
        # linear_kernel.f90:70-76 with order = 0 (the reference's default).
        xi = X[:, dims]
        order = 0.0
        R = np.zeros((n, n))
        for j in range(n):
            prod = xi[j:, :] * xi[j, :]
            R[j:, j] = np.sum((prod ** order) / params, axis=1)
        return R
    if op == CONSTANT:
        return np.full((n, n), float(params[0]))
    raise ValueError(op)


def kernel_R(kspec, theta, tens: Tensors):
    """k%R(X, R): evaluate the postfix kernel tree (kernel_module.f90:309-375)."""
    stack, p = [], 0
    for node in parse_kspec(kspec):
        if node[0] == "leaf":
            _, op, dims = node
            k = leaf_nparams(op, dims)
            params = leaf_transform(op, theta[p:p + k])
            p += k
            stack.append(leaf_R(op, dims, params, tens))
        else:
            b = stack.pop()
            a = stack.pop()
            stack.append(a + b if node[1] == SUM else a * b)
    assert len(stack) == 1
    return stack[0]


def compute_R(kspec, theta, noise, tens: Tensors):
    """gpr.f90:185-189: K = k(X, X) + nugget * identity."""
    K = kernel_R(kspec, theta, tens)
    return K + noise * np.eye(K.shape[0])


# --------------------------------------------------------------------------
# means (src/mean/*.f90) -- computed once per data set, passed to the engine
# --------------------------------------------------------------------------
def mean_vector(kind, X, y):
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n, d = X.shape
    if kind == "zero":
        return np.zeros(n)
    if kind == "constant":
        return np.full(n, float(np.sum(y)) / n)
    if kind in ("linear", "quadratic"):
        order = 1 if kind == "linear" else 2
        imin = int(np.argmin(y))              # Fortran minloc: first minimum
        xmin, ymin = X[imin].copy(), y[imin]
        a = X - xmin
        b = y - ymin
        for _ in range(order - 1):
            a = a * a
        aa = a.T @ a
        ab = (a.T @ b).reshape(d, 1)
        _, beta, info = lapack.dposv(aa, ab, lower=1)
        if info != 0:
            raise np.linalg.LinAlgError(f"dposv info={info}")
        beta = beta[:, 0]
        a = X - xmin
        if order == 2:
            a = a * a
        return a @ beta + ymin
    raise ValueError(kind)


# --------------------------------------------------------------------------
# likelihoods (likelihood.f90)
# --------------------------------------------------------------------------
def cholesky(K):
    """dpotrf('L') (likelihood.f90:145); returns (L, info)."""
    c, info = lapack.dpotrf(K, lower=1, clean=1)
    return c, int(info)


def log_determinant(L):
    """arith.f90:72-93: 2 * sum(log(L_ii)), accumulated in order."""
    s = 0.0
    for v in np.diag(L):
        s += math.log(v)
    return 2.0 * s


def potrs(L, b):
    x, info = lapack.dpotrs(L, np.asarray(b, dtype=np.float64), lower=1)
    return x


def loglik(kspec, theta, X, y, mu, likelihood, noise, optimise_noise, tens=None, want=False):
    """negative_log_likelihood -> log_likelihood -> ll_marginal / ll_concentrated.

    ``theta`` is the raw parameter vector (kernel params in tree order, then
    the linear noise value when ``optimise_noise``; gpr.f90:191-202).
    Returns ``(ll, info)`` or, with ``want=True``, a dict with ll, info,
    logdet, alpha, mean (concentrated) and sigma2 (concentrated).
    """
    theta = np.asarray(theta, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    nk = kernel_nparams(kspec)
    if optimise_noise:
        noise = float(theta[nk])
    if tens is None:
        tens = Tensors(X, need_cyclic=RBF_CYCLIC in list(kspec))
    K = compute_R(kspec, theta[:nk], noise, tens)
    n = K.shape[0]
    L, info = cholesky(K)
    out = {"info": info, "ll": float("nan"), "logdet": float("nan"), "alpha": None}
    if info != 0:
        return out if want else (float("nan"), info)
    logdet = log_determinant(L)
    out["logdet"] = logdet
    if likelihood == MARGINAL:
        r = y - np.asarray(mu, dtype=np.float64)
        alpha = potrs(L, r)
        ll = -0.5 * float(np.dot(r, alpha)) - 0.5 * logdet - 0.5 * n * LOG_TWOPI
    else:
        ry = potrs(L, y)
        ones = np.ones(n)
        r1 = potrs(L, ones)
        m = float(np.dot(ones, ry)) / float(np.dot(ones, r1))
        r = y - m
        alpha = potrs(L, r)
        s2 = float(np.dot(r, alpha)) / n
        with np.errstate(divide="ignore", invalid="ignore"):
            ll = -0.5 * n * float(np.log(s2)) - 0.5 * logdet   # Fortran log(0) = -Infinity
        out["mean"] = m
        out["sigma2"] = s2
    out["ll"] = ll
    out["alpha"] = alpha
    out["L"] = L
    return out if want else (ll, info)


# --------------------------------------------------------------------------
# analytic FP64 gradient (oracle for the adjoint) and central differences
# --------------------------------------------------------------------------
def kernel_R_and_grad(kspec, theta, tens: Tensors):
    """K(theta) and dK/dtheta_p for every kernel parameter p (dense, lower used).

    Leaf derivatives, with K_leaf the leaf matrix:
      rbf:      dK/dtheta_k = K_leaf * (-0.5 * l_k * D_k)        (l = exp(theta))
      periodic: dK/dtheta_k = K_leaf * ( 4.0 * l_k * P_k)        (l = exp(-2 theta))
      constant: dK/dtheta   = 1
      linear (order 0): dK/dtheta_k = exp(theta_k) * 1
    Products use the product rule, sums pass derivatives through.
    """
    stack, p = [], 0
    for node in parse_kspec(kspec):
        if node[0] == "leaf":
            _, op, dims = node
            k = leaf_nparams(op, dims)
            params = leaf_transform(op, theta[p:p + k])
            R = leaf_R(op, dims, params, tens)
            grads = {}
            for q in range(k):
                if op == RBF:
                    grads[p + q] = R * (-0.5 * params[q] * tens.D[dims[q]])
                elif op == PERIODIC:
                    grads[p + q] = R * (4.0 * params[q] * tens.P[dims[q]])
                elif op == RBF_CYCLIC:
                    grads[p + q] = R * (-0.5 * params[q] * tens.C[q])
                elif op == LINEAR:
                    grads[p + q] = np.full_like(R, math.exp(theta[p + q]))
                elif op == CONSTANT:
                    grads[p + q] = np.ones_like(R)
            p += k
            stack.append((R, grads))
        else:
            (Rb, gb) = stack.pop()
            (Ra, ga) = stack.pop()
            if node[1] == SUM:
                g = dict(ga)
                g.update(gb)
                stack.append((Ra + Rb, g))
            else:
                g = {q: v * Rb for q, v in ga.items()}
                g.update({q: Ra * v for q, v in gb.items()})
                stack.append((Ra * Rb, g))
    return stack[0]


def loglik_grad(kspec, theta, X, y, mu, likelihood, noise, optimise_noise, tens=None):
    """d logL / d theta = 1/2 tr((a a^T / s - K^-1) dK/dtheta), FP64.

    s = 1 (marginal) or sigma^2 (concentrated; envelope theorem over the
    profiled mean and variance).  The noise parameter (linear, gpr.f90:199-201)
    has dK/dnoise = I.
    """
    theta = np.asarray(theta, dtype=np.float64)
    nk = kernel_nparams(kspec)
    if optimise_noise:
        noise = float(theta[nk])
    if tens is None:
        tens = Tensors(X, need_cyclic=RBF_CYCLIC in list(kspec))
    res = loglik(kspec, theta, X, y, mu, likelihood, noise, optimise_noise, tens=tens, want=True)
    if res["info"] != 0:
        return res["ll"], None, res["info"]
    R, grads = kernel_R_and_grad(kspec, theta[:nk], tens)
    L = res["L"]
    n = L.shape[0]
    Kinv = lapack.dpotri(L, lower=1)[0]
    Kinv = np.tril(Kinv) + np.tril(Kinv, -1).T
    a = res["alpha"]
    s = 1.0 if likelihood == MARGINAL else res["sigma2"]
    W = np.outer(a, a) / s - Kinv
    g = np.zeros(len(theta))
    for q in range(nk):
        dK = np.tril(grads[q])
        dK = dK + np.tril(dK, -1).T
        g[q] = 0.5 * float(np.sum(W * dK))
    if optimise_noise:
        g[nk] = 0.5 * float(np.trace(W))
    return res["ll"], g, 0


def central_fd(kspec, theta, X, y, mu, likelihood, noise, optimise_noise, rel=1e-6, tens=None):
    """Central differences with h = rel * |theta_p| (h = rel when theta_p = 0)."""
    theta = np.asarray(theta, dtype=np.float64)
    if tens is None:
        tens = Tensors(X, need_cyclic=RBF_CYCLIC in list(kspec))
    g = np.zeros(len(theta))
    for p in range(len(theta)):
        h = rel * abs(theta[p]) if theta[p] != 0 else rel
        tp, tm = theta.copy(), theta.copy()
        tp[p] += h
        tm[p] -= h
        lp, ip = loglik(kspec, tp, X, y, mu, likelihood, noise, optimise_noise, tens=tens)
        lm, im = loglik(kspec, tm, X, y, mu, likelihood, noise, optimise_noise, tens=tens)
        g[p] = (lp - lm) / (tp[p] - tm[p])
    return g


# --------------------------------------------------------------------------
# independent cross-checks used to pin the restatement
# --------------------------------------------------------------------------
def pairwise_k(op, dims, params, xi, xj):
    """The reference's pairwise ``k`` functions (rbf_kernel.f90:73-91,
    periodic_kernel.f90:73-91 -- NOTE the pairwise periodic form uses
    sin(diff), not sin(diff/2), so it is NOT used to pin the periodic R)."""
    diff = xi[dims] - xj[dims]
    if op == RBF:
        return math.exp(-0.5 * float(np.sum(params * diff * diff)))
    if op == PERIODIC:
        s = np.sin(diff)
        return math.exp(-2.0 * float(np.sum(params * s * s)))
    raise ValueError(op)


def cholesky_python(K):
    """Unblocked column Cholesky in pure Python/numpy (independent of LAPACK)."""
    A = np.array(K, dtype=np.float64)
    n = A.shape[0]
    L = np.zeros_like(A)
    for j in range(n):
        s = A[j, j] - float(np.dot(L[j, :j], L[j, :j]))
        if not s > 0.0:
            return L, j + 1
        L[j, j] = math.sqrt(s)
        if j + 1 < n:
            L[j + 1:, j] = (A[j + 1:, j] - L[j + 1:, :j] @ L[j, :j]) / L[j, j]
    return L, 0


def loglik_grad_columns(kspec, theta, X, y, mu, likelihood, noise, optimise_noise):
    """Memory-light FP64 gradient for large N: the same formula as
    ``loglik_grad`` (1/2 sum_ij W_ij dK_ij/dtheta, W = a a^T / s - K^-1), with
    dK/dtheta formed one column at a time (rows i >= j, weight 2 off the
    diagonal) instead of one dense matrix per parameter."""
    theta = np.asarray(theta, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    n, d = X.shape
    nk = kernel_nparams(kspec)
    if optimise_noise:
        noise = float(theta[nk])
    tens = Tensors(X, lazy=True)
    res = loglik(kspec, theta, X, y, mu, likelihood, noise, optimise_noise, tens=tens, want=True)
    if res["info"] != 0:
        return res["ll"], None, res["info"]
    L = res["L"]
    Kinv = lapack.dpotri(L, lower=1)[0]
    a = res["alpha"]
    s = 1.0 if likelihood == MARGINAL else res["sigma2"]
    nodes = parse_kspec(kspec)
    # leaf parameter offsets and transformed parameters
    leaves, p = [], 0
    for node in nodes:
        if node[0] == "leaf":
            k = leaf_nparams(node[1], node[2])
            leaves.append((p, leaf_transform(node[1], theta[p:p + k])))
            p += k
    g = np.zeros(len(theta))
    xt = X.T
    cyc = np.arange(2, d, 3)
    for j in range(n):
        w = a[j:] * a[j] / s - Kinv[j:, j]
        w[1:] *= 2.0
        diff = xt[:, j:] - xt[:, j:j + 1]
        wrapped = diff.copy()
        c = wrapped[cyc]
        aa = np.abs(c) + PI
        wrapped[cyc] = np.where(c == 0.0, 0.0, np.sign(c) * ((aa - np.trunc(aa / TWOPI) * TWOPI) - PI))
        P = np.sin(np.sqrt(diff * diff) / 2.0) ** 2
        vals, derivs, li = [], [], 0
        stack = []
        for node in nodes:
            if node[0] == "leaf":
                op, dims = node[1], node[2]
                p0, prm = leaves[li]
                li += 1
                m = len(w)
                if op == RBF:
                    t = prm[:, None] * diff[dims] ** 2
                    v = np.exp(-0.5 * t.sum(axis=0))
                    dv = [(p0 + q, v * (-0.5 * t[q])) for q in range(len(dims))]
                elif op == RBF_CYCLIC:
                    t = prm[:, None] * wrapped[dims] ** 2
                    v = np.exp(-0.5 * t.sum(axis=0))
                    dv = [(p0 + q, v * (-0.5 * t[q])) for q in range(len(dims))]
                elif op == PERIODIC:
                    t = prm[:, None] * P[dims]
                    v = np.exp(-2.0 * t.sum(axis=0))
                    dv = [(p0 + q, v * (4.0 * t[q])) for q in range(len(dims))]
                elif op == LINEAR:
                    v = np.full(m, float(np.sum(1.0 / prm)))
                    dv = [(p0 + q, np.full(m, 1.0 / prm[q])) for q in range(len(dims))]
                else:
                    v = np.full(m, float(prm[0]))
                    dv = [(p0, np.ones(m))]
                stack.append((v, dv))
            else:
                vb, db = stack.pop()
                va, da = stack.pop()
                if node[1] == SUM:
                    stack.append((va + vb, da + db))
                else:
                    stack.append((va * vb, [(q, x * vb) for q, x in da] + [(q, va * x) for q, x in db]))
        _, dK = stack[0]
        for q, x in dK:
            g[q] += 0.5 * float(np.dot(w, x))
        if optimise_noise:
            g[nk] += 0.5 * (a[j] * a[j] / s - Kinv[j, j])
    return res["ll"], g, 0
