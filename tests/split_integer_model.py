"""A numpy model of the tensor-core factorisation's arithmetic (test
infrastructure, CPU only).

It restates the engine's split-integer blocked Cholesky so that the scheme's
accuracy can be checked against LAPACK without a GPU:

* 128-wide panels; the work inside a panel (its diagonal block's Cholesky
  and the panel solve) in FP64 (LAPACK here; on the GPU the FP64 32-column
  quarters with tensor-core couplings between them);
* row scales e_i with sqrt(K_ii) (1 + 2^-20) < 2^e_i;
* each finished panel column entry as a 55-bit fixed point in its row scale,
  split into 7 balanced base-256 digits;
* the trailing update from the digit products of levels p + q <= 6, each
  level an exact integer sum, gathered as W = hi 2^24 + lo and accumulated
  exactly across panels;
* one rounding per element when a block column becomes the panel:
  K_ij - W_ij 2^(e_i + e_j - 62).

The GPU tests check the kernels against the oracle; this checks the scheme.
"""
import math

import numpy as np
from scipy import linalg as sla
from scipy.linalg import lapack

NB = 128
LOG_TWOPI = math.log(2.0 * math.pi)


def row_scales(A):
    """smallest e_i with sqrt(A_ii) (1 + 2^-20) < 2^e_i (frexp)."""
    _, E = np.frexp(np.sqrt(np.diag(A)) * (1.0 + 2.0 ** -20))
    return E.astype(np.int64)


def digits(x, e):
    """(7, m, k) balanced digits of round(x 2^(55 - e_row)), top digit first;
    rounding half away from zero as the engine does."""
    y = np.ldexp(np.abs(x), (55 - e)[:, None])
    F = (np.sign(x) * np.floor(y + 0.5)).astype(np.int64)
    G = F + 0x808080808080
    D = np.empty((7,) + F.shape, dtype=np.int64)
    D[0] = G >> 48
    for p in range(1, 7):
        D[p] = ((G >> (8 * (6 - p))) & 0xFF) - 128
    return D


def level_hi_lo(Da, Db, levels=7):
    """W = sum_{p + q < levels} (Da_p Db_q^T) 2^(8 (12 - p - q) - 48) as
    hi 2^24 + lo (the engine keeps 7 levels).  Each level sum is an integer
    below 2^24, so float64 matrix products are exact."""
    Fa, Fb = Da.astype(np.float64), Db.astype(np.float64)
    S = []
    for lev in range(7):
        if lev >= levels:
            S.append(np.zeros((Da.shape[1], Db.shape[1]), dtype=np.int64))
            continue
        acc = np.zeros((Da.shape[1], Db.shape[1]))
        for p in range(lev + 1):
            acc += Fa[p] @ Fb[lev - p].T
        S.append(acc.astype(np.int64))
    low = S[4] * 65536 + S[5] * 256 + S[6]
    hi = S[0] * 16777216 + S[1] * 65536 + S[2] * 256 + S[3] + (low >> 24)
    return hi, low & 0xFFFFFF


def factor(K, levels=7):
    """Lower factor of the SPD matrix K by the split-integer scheme keeping
    the digit-product levels below `levels`; returns (L, info) with LAPACK's
    info convention."""
    n = K.shape[0]
    nc = -(-n // NB) * NB
    A = np.eye(nc)
    A[:n, :n] = np.tril(K)
    e = row_scales(A)
    acc_hi = np.zeros((nc, nc), dtype=np.int64)
    acc_lo = np.zeros((nc, nc), dtype=np.int64)
    for c0 in range(0, nc, NB):
        c1 = c0 + NB
        if c0 > 0:  # the exact sums of the earlier panels, one rounding each
            w = acc_hi[c0:, c0:c1].astype(np.float64) * 16777216.0 + acc_lo[c0:, c0:c1]
            A[c0:, c0:c1] -= np.ldexp(w, e[c0:, None] + e[None, c0:c1] - 62)
        Lpp, info = lapack.dpotrf(A[c0:c1, c0:c1], lower=1, clean=1)
        if info != 0:
            return None, int(info) + c0
        A[c0:c1, c0:c1] = Lpp
        if c1 < nc:
            A[c1:, c0:c1] = sla.solve_triangular(Lpp, A[c1:, c0:c1].T, lower=True).T
            D = digits(A[c1:, c0:c1], e[c1:])
            hi, lo = level_hi_lo(D, D, levels)
            acc_hi[c1:, c1:] += hi
            acc_lo[c1:, c1:] += lo
            acc_hi[c1:, c1:] += acc_lo[c1:, c1:] >> 24
            acc_lo[c1:, c1:] &= 0xFFFFFF
    return np.tril(A[:n, :n]), 0


def loglik_from_factor(L, y, mu, likelihood):
    """The likelihoods of likelihood.f90:161-253 from a factor (marginal = 0,
    concentrated = 1), as the oracle forms them."""
    n = L.shape[0]
    logdet = 2.0 * float(np.sum(np.log(np.diag(L))))

    def solve(b):
        return lapack.dpotrs(L, np.asarray(b, dtype=np.float64), lower=1)[0]

    if likelihood == 0:
        r = y - mu
        return -0.5 * float(r @ solve(r)) - 0.5 * logdet - 0.5 * n * LOG_TWOPI
    ones = np.ones(n)
    m = float(ones @ solve(y)) / float(ones @ solve(ones))
    r = y - m
    s2 = float(r @ solve(r)) / n
    return -0.5 * n * math.log(s2) - 0.5 * logdet


def couple(T, X, ex, Y, ey, levels=7):
    """T -= round(sum_k X_ik Y_jk) from digit planes (the couplings inside a
    panel): the exact level sums converted with one rounding, then
    subtracted.  X: rows of T in their scales ex; Y: the coupled columns' L
    rows in their scales ey."""
    hi, lo = level_hi_lo(digits(X, ex), digits(Y, ey), levels)
    w = hi.astype(np.float64) * 16777216.0 + lo
    T -= np.ldexp(w, ex[:, None] + ey[None, :] - 62)


def panel_solve(B, Lqq, eb, eq, pieces=2, levels=7):
    """X Lqq^T = B for the rows below a 32 x 32 diagonal block: FP64
    substitution in pieces of 32 / pieces columns, the later pieces coupled
    to the earlier ones on digit planes.  pieces = 2: the engine's two
    halves, one coupling; pieces = 4: 8-column pieces with couplings
    0 -> 1, (0, 1) -> (2, 3), 2 -> 3."""
    X = B.copy()
    w = 32 // pieces

    def solve(p):
        c = slice(p * w, (p + 1) * w)
        X[:, c] = sla.solve_triangular(Lqq[c, c], X[:, c].T, lower=True).T

    if pieces == 2:
        solve(0)
        couple(X[:, 16:], X[:, :16], eb, Lqq[16:, :16], eq[16:], levels)
        solve(1)
    elif pieces == 4:
        solve(0)
        couple(X[:, 8:16], X[:, :8], eb, Lqq[8:16, :8], eq[8:16], levels)
        solve(1)
        couple(X[:, 16:], X[:, :16], eb, Lqq[16:, :16], eq[16:], levels)
        solve(2)
        couple(X[:, 24:], X[:, 16:24], eb, Lqq[24:, 16:24], eq[24:], levels)
        solve(3)
    else:
        raise ValueError(pieces)
    return X


def factor_quarters(K, pieces=2, levels=7):
    """As `factor`, with the panel worked as the engine works it: four
    32-column quarters (FP64 diagonal factor, panel solve in pieces) and the
    digit-plane couplings quarter 0 -> 1, half 0 -> half 1, quarter 2 -> 3."""
    n = K.shape[0]
    nc = -(-n // NB) * NB
    A = np.eye(nc)
    A[:n, :n] = np.tril(K)
    e = row_scales(A)
    acc_hi = np.zeros((nc, nc), dtype=np.int64)
    acc_lo = np.zeros((nc, nc), dtype=np.int64)
    for c0 in range(0, nc, NB):
        c1 = c0 + NB
        if c0 > 0:
            w = acc_hi[c0:, c0:c1].astype(np.float64) * 16777216.0 + acc_lo[c0:, c0:c1]
            A[c0:, c0:c1] -= np.ldexp(w, e[c0:, None] + e[None, c0:c1] - 62)
        for q in range(4):
            a = c0 + 32 * q
            b = a + 32
            if q == 1:
                couple(A[a:, a:b], A[a:, c0:a], e[a:], A[a:b, c0:a], e[a:b], levels)
            elif q == 2:
                couple(A[a:, a:c1], A[a:, c0:a], e[a:], A[a:c1, c0:a], e[a:c1], levels)
            elif q == 3:
                couple(A[a:, a:b], A[a:, c0 + 64:a], e[a:], A[a:b, c0 + 64:a], e[a:b], levels)
            Lqq, info = lapack.dpotrf(A[a:b, a:b], lower=1, clean=1)
            if info != 0:
                return None, int(info) + a
            A[a:b, a:b] = Lqq
            if b < nc:
                A[b:, a:b] = panel_solve(A[b:, a:b], Lqq, e[b:], e[a:b], pieces, levels)
        if c1 < nc:
            D = digits(A[c1:, c0:c1], e[c1:])
            hi, lo = level_hi_lo(D, D, levels)
            acc_hi[c1:, c1:] += hi
            acc_lo[c1:, c1:] += lo
            acc_hi[c1:, c1:] += acc_lo[c1:, c1:] >> 24
            acc_lo[c1:, c1:] &= 0xFFFFFF
    return np.tril(A[:n, :n]), 0
