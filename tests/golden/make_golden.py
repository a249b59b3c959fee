"""Generate the golden fixtures under tests/golden/ from the CPU oracle.

Run in the development container (it reads the reference's example CSVs,
which do not travel to the GPU machine); ``--examples-dir`` is the
``examples`` folder of a FEREBUS-v7 checkout:

    python tests/golden/make_golden.py --examples-dir <FEREBUS-v7>/examples

Each ``<case>.npz`` holds the inputs (X, y, mu, kspec, likelihood, noise,
optimise_noise), a few parameter vectors, and for each of them:

* ``ll`` -- the oracle's value (OpenBLAS dpotrf/dpotrs, the reference's LAPACK
  path), with ``info`` and ``logdet``, and ``alpha0`` for the first vector;
* ``ll_exact`` -- the same formulas in extended precision
  (``oracle/exact.py``, 64-bit significand on x86-64), the value FP64 codes
  are measured against;
* ``fp64_err`` -- the FP64 error scale: the largest |ll' - ll_exact| over
  OpenBLAS, an independent LAPACK (MKL through torch) and OpenBLAS on eight
  random symmetric 4-ulp perturbations of K (the backward error any FP64
  evaluation of K and its Cholesky carries);
* ``spread`` -- the largest |ll' - ll| over MKL and three such perturbations
  (kept for reference).

``full_size.json`` holds the same quantities for the two ill-conditioned
benchmark shapes at their full size (water-like N=500, methanol-like
N=2000), with their targets y; the tests regenerate the features X from the
seeded generators and check them against the stored SHA-256 digest.

Example data (examples/*/..._TRAINING_SET.csv of FEREBUS-v7) are stored as
row subsets of the feature columns and the ``iqa`` target only.
"""
from __future__ import annotations

import argparse
import csv
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "ferebus-v7_gb300"))

from oracle import gpr_oracle as O  # noqa: E402
from oracle import exact as E  # noqa: E402
from fgpu import synth  # noqa: E402
from fgpu.kernel_spec import build_kspec  # noqa: E402


def read_csv(path, nrows=None):
    with open(path) as f:
        rd = csv.reader(f)
        head = next(rd)
        fcols = [i for i, h in enumerate(head) if h.startswith("f")]
        tcol = head.index("iqa")
        X, y = [], []
        for k, row in enumerate(rd):
            if nrows is not None and k >= nrows:
                break
            X.append([float(row[i]) for i in fcols])
            y.append(float(row[tcol]))
    return np.array(X), np.array(y)


def mkl_ll(K, y, mu, likelihood):
    import torch
    Kt = torch.tensor(np.tril(K) + np.tril(K, -1).T)
    L, info = torch.linalg.cholesky_ex(Kt)
    if int(info) != 0:
        return float("nan")
    n = K.shape[0]
    logdet = 2.0 * float(torch.log(torch.diagonal(L)).sum())
    if likelihood == 0:
        r = torch.tensor(y - mu).reshape(n, 1)
        a = torch.cholesky_solve(r, L)
        return float(-0.5 * (r * a).sum() - 0.5 * logdet - 0.5 * n * O.LOG_TWOPI)
    yt = torch.tensor(y).reshape(n, 1)
    one = torch.ones(n, 1, dtype=torch.float64)
    ry = torch.cholesky_solve(yt, L)
    r1 = torch.cholesky_solve(one, L)
    m = float(ry.sum() / r1.sum())
    r = yt - m
    a = torch.cholesky_solve(r, L)
    s2 = float((r * a).sum()) / n
    return -0.5 * n * np.log(s2) - 0.5 * logdet


def ll_from_K(K, y, mu, likelihood):
    """The oracle's likelihood formula on a given K (OpenBLAS dpotrf/dpotrs)."""
    n = K.shape[0]
    L, info = O.cholesky(K)
    if info != 0:
        return float("nan")
    logdet = O.log_determinant(L)
    if likelihood == 0:
        r = y - mu
        return -0.5 * float(r @ O.potrs(L, r)) - 0.5 * logdet - 0.5 * n * O.LOG_TWOPI
    ry, r1 = O.potrs(L, y), O.potrs(L, np.ones(n))
    m = float(ry.sum()) / float(r1.sum())
    r = y - m
    return -0.5 * n * np.log(float(r @ O.potrs(L, r)) / n) - 0.5 * logdet


def noise_floor(K, y, mu, likelihood, ll, rng, trials=3):
    """Largest |ll' - ll| over an independent LAPACK (MKL) and a few random
    symmetric perturbations K_ij (1 + e_ij), |e_ij| <= 4 u -- the backward
    error any FP64 evaluation of K and its Cholesky carries."""
    u = np.finfo(np.float64).eps / 2
    worst = abs(mkl_ll(K, y, mu, likelihood) - ll)
    Ks = np.tril(K) + np.tril(K, -1).T
    for _ in range(trials):
        E = rng.uniform(-4 * u, 4 * u, size=K.shape)
        E = np.tril(E) + np.tril(E, -1).T
        lp = ll_from_K(Ks * (1.0 + E), y, mu, likelihood)
        if np.isfinite(lp):
            worst = max(worst, abs(lp - ll))
    return worst


def fp64_error_scale(K, y, mu, likelihood, ll_ob, ll_exact, rng, trials=8):
    """Largest |ll' - ll_exact| over OpenBLAS, MKL and OpenBLAS on `trials`
    random symmetric perturbations K_ij (1 + e_ij), |e_ij| <= 4 u."""
    u = np.finfo(np.float64).eps / 2
    worst = max(abs(ll_ob - ll_exact), abs(mkl_ll(K, y, mu, likelihood) - ll_exact))
    Ks = np.tril(K) + np.tril(K, -1).T
    for _ in range(trials):
        Ep = rng.uniform(-4 * u, 4 * u, size=K.shape)
        Ep = np.tril(Ep) + np.tril(Ep, -1).T
        lp = ll_from_K(Ks * (1.0 + Ep), y, mu, likelihood)
        if np.isfinite(lp):
            worst = max(worst, abs(lp - ll_exact))
    return worst


def make_case(name, X, y, mean, kspec, likelihood, noise=1e-10, optimise_noise=False, thetas=None,
              seed=0, lo=1e-3, hi=1.0):
    rng = np.random.default_rng(seed)
    nk = O.kernel_nparams(kspec)
    mu = O.mean_vector(mean, X, y)
    if thetas is None:
        thetas = rng.uniform(lo, hi, size=(4, nk + (1 if optimise_noise else 0)))
        if optimise_noise:
            thetas[:, nk] = 10.0 ** rng.uniform(-12, -6, size=4)
    tens = O.Tensors(X, need_cyclic=O.RBF_CYCLIC in kspec)
    out = {k: [] for k in ("ll", "info", "logdet", "spread", "ll_exact", "fp64_err")}
    alpha0 = None
    for t, th in enumerate(thetas):
        r = O.loglik(kspec, th, X, y, mu, likelihood, noise, optimise_noise, tens=tens, want=True)
        out["ll"].append(r["ll"])
        out["info"].append(r["info"])
        out["logdet"].append(r["logdet"])
        if r["info"] == 0:
            nz = float(th[nk]) if optimise_noise else noise
            K = O.compute_R(kspec, th[:nk], nz, tens)
            out["spread"].append(noise_floor(K, y, mu, likelihood, r["ll"], rng))
            ex = E.loglik_ld(kspec, th, X, y, mu, likelihood, noise, optimise_noise)[0]
            out["ll_exact"].append(ex)
            out["fp64_err"].append(fp64_error_scale(K, y, mu, likelihood, r["ll"], ex, rng))
        else:
            out["spread"].append(0.0)
            out["ll_exact"].append(float("nan"))
            out["fp64_err"].append(0.0)
        if t == 0:
            alpha0 = r["alpha"] if r["alpha"] is not None else np.zeros(len(y))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, X=X, y=y, mu=mu, kspec=np.array(kspec, dtype=np.int32), likelihood=likelihood,
                        noise=noise, optimise_noise=int(optimise_noise), thetas=np.array(thetas),
                        ll=np.array(out["ll"]), info=np.array(out["info"], dtype=np.int32),
                        logdet=np.array(out["logdet"]), spread=np.array(out["spread"]), alpha0=alpha0,
                        ll_exact=np.array(out["ll_exact"]), fp64_err=np.array(out["fp64_err"]))
    print(f"{name:24s} N={len(y):5d} d={X.shape[1]:3d} info={out['info']} rel_fp64_err="
          f"{['%.1e' % (s / max(abs(l), 1e-300)) for s, l in zip(out['fp64_err'], out['ll_exact'])]}")


def digest(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def make_full_size():
    """full_size.json: the ill-conditioned benchmark shapes at full size."""
    import json
    res = {}
    for key, p in (("water_like_500", synth.config1()), ("methanol_like_2000", synth.config2())):
        rng = np.random.default_rng(31)
        mu = O.mean_vector(p.mean, p.X, p.y)
        th = p.thetas(3, seed=5)
        tens = O.Tensors(p.X, lazy=True)
        nk = O.kernel_nparams(p.kspec)
        rows = []
        for t in th:
            K = O.compute_R(p.kspec, t[:nk], p.noise, tens)
            ob = ll_from_K(K, p.y, mu, p.likelihood)
            ex = E.loglik_ld(p.kspec, t, p.X, p.y, mu, p.likelihood, p.noise, False)[0]
            err = fp64_error_scale(K, p.y, mu, p.likelihood, ob, ex, rng)
            rows.append({"theta": [float(v) for v in t], "ll_openblas": ob, "ll_exact": ex, "fp64_err": err})
            print(f"{key} rel_fp64_err={err / abs(ex):.2e} rel_openblas_err={abs(ob - ex) / abs(ex):.2e}")
        # y is stored: the generator forms it through a BLAS product, whose
        # last bits differ between machines; X is regenerated and checked
        res[key] = {"N": p.N, "d": p.d, "X_sha256": digest(p.X), "y": [float(v) for v in p.y], "mean": p.mean,
                    "thetas": rows}
    with open(os.path.join(HERE, "full_size.json"), "w") as f:
        json.dump(res, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--examples-dir", required=True, help="the examples folder of a FEREBUS-v7 checkout")
    ap.add_argument("--full-size-only", action="store_true")
    a = ap.parse_args()
    make_full_size()
    if a.full_size_only:
        return
    ex = a.examples_dir
    R = O.RBF
    # --- the reference's shipped example data sets ---------------------------------
    X, y = read_csv(os.path.join(ex, "WATER", "WATER_O1_TRAINING_SET.csv"))
    ks, _ = build_kspec("k1*k2", {"k1": {"type": "rbf"}, "k2": {"type": "periodic", "active_dimensions": [3]}}, 3)
    make_case("water_O1_rbf_x_per", X, y, "constant", ks, 0, seed=1)
    X, y = read_csv(os.path.join(ex, "WATER", "WATER_H2_TRAINING_SET.csv"))
    ks, _ = build_kspec("k1+k2", {"k1": {"type": "rbf", "active_dimensions": [1, 2]},
                                 "k2": {"type": "periodic", "active_dimensions": [3]}}, 3)
    make_case("water_H2_rbf_plus_per", X, y, "linear", ks, 0, seed=2)
    X, y = read_csv(os.path.join(ex, "AMMONIA", "AMMONIA_N1_TRAINING_SET.csv"))
    make_case("ammonia_N1_rbf", X, y, "constant", [R, 6, 1, 2, 3, 4, 5, 6], 0, seed=3)
    X, y = read_csv(os.path.join(ex, "METHANOL", "METHANOL_C1_TRAINING_SET.csv"), nrows=400)
    make_case("methanol_C1_rbf_q", X, y, "quadratic", [R, 12] + list(range(1, 13)), 0, seed=4)
    X, y = read_csv(os.path.join(ex, "NMA", "NMA_C1_TRAINING_SET.csv"), nrows=300)
    make_case("nma_C1_rbf_conc", X, y, "constant", [R, 30] + list(range(1, 31)), 1, seed=5, hi=3.0)
    X, y = read_csv(os.path.join(ex, "GLYCINE", "GLYCINE_C1_TRAINING_SET.csv"), nrows=300)
    make_case("glycine_C1_rbf", X, y, "zero", [R, 51] + list(range(1, 52)), 0, seed=6, hi=3.0)
    # --- seeded synthetic stand-ins for the benchmark configs (reduced N) -----------
    p = synth.config1(200)
    make_case("syn_c1_water_like", p.X, p.y, p.mean, p.kspec, p.likelihood, seed=11)
    p = synth.config2(257)
    make_case("syn_c2_methanol_like", p.X, p.y, p.mean, p.kspec, p.likelihood, seed=12)
    p = synth.config3(321)
    make_case("syn_c3_glycine_like", p.X, p.y, p.mean, p.kspec, p.likelihood, seed=13)
    p = synth.config4(natoms=2, nmin=60, nmax=140)[1]
    make_case("syn_c4_atom_linear_mean", p.X, p.y, p.mean, p.kspec, p.likelihood, seed=14)
    p = synth.config5(190)
    make_case("syn_c5_noise_quadratic", p.X, p.y, p.mean, p.kspec, p.likelihood, optimise_noise=True, seed=15)
    # --- kernel families and compositions the path supports -------------------------
    rng = np.random.default_rng(99)
    X = np.column_stack([rng.normal(2.0, 0.1, 130), rng.normal(1.9, 0.1, 130), rng.uniform(-3.1, 3.1, 130),
                         rng.normal(2.0, 0.1, 130), rng.normal(1.8, 0.1, 130), rng.uniform(-3.1, 3.1, 130)])
    y = np.sin(X[:, 0]) + np.cos(X[:, 2]) + 0.1 * X[:, 4] + rng.normal(0, 1e-3, 130)
    make_case("cyclic_rbf_all_dims", X, y, "constant", [O.RBF_CYCLIC, 6, 1, 2, 3, 4, 5, 6], 0, seed=21)
    ks, _ = build_kspec("k1*k2*k3+k4", {"k1": {"type": "rbf", "active_dimensions": [1, 2]},
                                         "k2": {"type": "periodic", "active_dimensions": [3, 6]},
                                         "k3": {"type": "rbf", "active_dimensions": [4, 5]},
                                         "k4": {"type": "rbf", "active_dimensions": [1]}}, 6)
    make_case("composite_prod_sum", X, y, "constant", ks, 0, seed=22)
    ks, _ = build_kspec("k1+0.5", {"k1": {"type": "rbf"}}, 6)
    make_case("rbf_plus_constant", X, y, "constant", ks, 0, seed=23)
    ks, _ = build_kspec("(k1+k2)*k3", {"k1": {"type": "rbf", "active_dimensions": [1, 2, 4]},
                                        "k2": {"type": "linear", "active_dimensions": [5]},
                                        "k3": {"type": "periodic", "active_dimensions": [3]}}, 6)
    make_case("linear_in_composite_conc", X, y, "constant", ks, 1, seed=24)
    # a non-positive-definite K: duplicated rows, zero nugget -> info > 0
    Xd = np.vstack([X[:40], X[:40]])
    yd = np.concatenate([y[:40], y[:40]])
    make_case("duplicate_rows_not_pd", Xd, yd, "constant", [R, 6, 1, 2, 3, 4, 5, 6], 0, noise=0.0, seed=25,
              thetas=np.array([[-2.0] * 6, [0.5] * 6]))


if __name__ == "__main__":
    main()
