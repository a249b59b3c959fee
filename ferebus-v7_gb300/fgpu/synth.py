"""Seeded synthetic training sets with the shapes of the five benchmark configs.

The reference trains on CSV files of molecular features; there is no public
data set for these sizes, so seeded generators with the stated shapes and value
distributions stand in for them.  Seeds are ``20261203 + config index``
(``numpy.random.default_rng``).

=====  ======  =====  ==========================================  ===================
cfg    N       d      kernel                                      likelihood / mean
=====  ======  =====  ==========================================  ===================
1      500     3      rbf(1,2) + periodic(3)                      marginal / constant
2      2000    12     rbf(1..9) + periodic(10..12)                marginal / constant
3      4000    24     rbf(17 non-dihedral) + periodic(6,9,..,24)  concentrated
4      33 x U{500..6000}, 93   rbf + periodic(6,9,..,93)          marginal / linear
5      10000   30     rbf + periodic(dihedrals)                   marginal / quadratic, optimise_noise
=====  ======  =====  ==========================================  ===================
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .kernel_spec import PERIODIC, RBF, SUM

SEED0 = 20261203


@dataclass
class Problem:
    """One GPR training problem: data, kernel spec, likelihood and swarm shape."""
    name: str
    X: np.ndarray            # (N, d) float64, C-contiguous rows are points
    y: np.ndarray            # (N,)
    mean: str                # zero | constant | linear | quadratic
    kspec: list
    likelihood: int          # 0 marginal, 1 concentrated
    noise: float = 1e-10
    optimise_noise: bool = False
    swarm: int = 20
    iterations: int = 50
    theta_lo: float = 1e-3
    theta_hi: float = 1.0
    extra: dict = field(default_factory=dict)

    @property
    def N(self):
        return self.X.shape[0]

    @property
    def d(self):
        return self.X.shape[1]

    @property
    def ntheta(self):
        from .kernel_spec import nparams
        return nparams(self.kspec) + (1 if self.optimise_noise else 0)

    def thetas(self, count, seed=0):
        """Particle positions drawn uniformly from the search box."""
        rng = np.random.default_rng(SEED0 + 1000 + seed)
        nk = self.ntheta - (1 if self.optimise_noise else 0)
        th = rng.uniform(self.theta_lo, self.theta_hi, size=(count, self.ntheta))
        if self.optimise_noise:
            # The reference's noise parameter is linear in [1e-12, 1e-6]
            # (src/model/gpr/gpr.f90:221-245); draw log10-noise uniformly in
            # [-12, -6] and map to the linear value the engine consumes.
            th[:, nk] = 10.0 ** rng.uniform(-12.0, -6.0, size=count)
        return th


def _rbf_per_spec(d, per_dims):
    """rbf over the non-periodic dims + periodic over ``per_dims`` (1-based)."""
    per = sorted(per_dims)
    rbf = [i for i in range(1, d + 1) if i not in set(per)]
    spec = [RBF, len(rbf)] + rbf
    if per:
        spec += [PERIODIC, len(per)] + per + [SUM]
    return spec


def _rff(rng, X, M, noise_sd):
    d = X.shape[1]
    w = rng.normal(0.0, 1.0, size=(M, d))
    b = rng.uniform(0.0, 2 * np.pi, size=M)
    a = rng.normal(0.0, np.sqrt(1.0 / M), size=M)
    return np.cos(X @ w.T + b) @ a + rng.normal(0.0, noise_sd, size=X.shape[0])


def _features_c2(rng, n, d, dihedral_dims):
    """Bond-like N(2.0,0.1) / angle-like U(1.7,2.1) / dihedral U(-pi,pi) columns."""
    X = np.empty((n, d))
    dih = set(dihedral_dims)
    for j in range(d):
        f = j + 1
        if f in dih:
            X[:, j] = rng.uniform(-np.pi, np.pi, size=n)
        elif (j % 3) == 0 or j < 6:
            X[:, j] = rng.normal(2.0, 0.1, size=n)
        else:
            X[:, j] = rng.uniform(1.7, 2.1, size=n)
    return X


def config1(n=500):
    rng = np.random.default_rng(SEED0 + 1)
    X = np.empty((n, 3))
    X[:, 0] = rng.normal(1.81, 0.05, n)
    X[:, 1] = rng.normal(1.81, 0.05, n)
    X[:, 2] = rng.normal(1.82, 0.08, n)
    y = (-75.4 + 0.3 * np.sin(2.0 * X[:, 0]) + 0.2 * (X[:, 1] - 1.81) ** 2
         + 0.1 * np.sin(X[:, 2]) * np.cos(X[:, 0]) + rng.normal(0.0, 1e-4, n))
    spec = [RBF, 2, 1, 2, PERIODIC, 1, 3, SUM]
    return Problem("water-O1-like N=%d d=3" % n, X, y, "constant", spec, 0,
                   swarm=20, iterations=50)


def config2(n=2000):
    rng = np.random.default_rng(SEED0 + 2)
    X = np.empty((n, 12))
    X[:, 0:6] = rng.normal(2.0, 0.1, size=(n, 6))
    X[:, 6:9] = rng.uniform(1.7, 2.1, size=(n, 3))
    X[:, 9:12] = rng.uniform(-np.pi, np.pi, size=(n, 3))
    y = _rff(rng, X, 64, np.sqrt(1e-5))
    spec = [RBF, 9] + list(range(1, 10)) + [PERIODIC, 3, 10, 11, 12, SUM]
    return Problem("methanol-like N=%d d=12" % n, X, y, "constant", spec, 0,
                   swarm=50, iterations=100)


def config3(n=4000):
    rng = np.random.default_rng(SEED0 + 3)
    d = 24
    dih = list(range(6, d + 1, 3))          # f6, f9, ..., f24 (7 dihedrals)
    X = np.empty((n, d))
    for j in range(d):
        if (j + 1) in dih:
            X[:, j] = rng.uniform(-np.pi, np.pi, size=n)
        else:
            X[:, j] = rng.normal(2.2, 0.15, size=n)
    y = _rff(rng, X, 128, np.sqrt(1e-5))
    return Problem("glycine-like N=%d d=24" % n, X, y, "constant", _rbf_per_spec(d, dih), 1,
                   swarm=40, iterations=100)


def config4(natoms=33, nmin=500, nmax=6000, scale=1.0):
    """Ragged multi-atom batch; ``scale`` shrinks every N (for tests)."""
    rng = np.random.default_rng(SEED0 + 4)
    d = 93
    dih = list(range(6, d + 1, 3))          # 30 dihedrals
    sizes = rng.integers(nmin, nmax + 1, size=natoms)
    probs = []
    for a, na in enumerate(sizes):
        na = max(2, int(round(na * scale)))
        X = _features_c2(rng, na, d, dih)
        y = _rff(rng, X, 64, np.sqrt(1e-5))
        probs.append(Problem("atom%d N=%d d=93" % (a + 1, na), X, y, "linear",
                             _rbf_per_spec(d, dih), 0, swarm=30, iterations=60))
    return probs


def config5(n=10000):
    rng = np.random.default_rng(SEED0 + 5)
    d = 30
    dih = list(range(6, d + 1, 3))
    X = _features_c2(rng, n, d, dih)
    y = _rff(rng, X, 64, np.sqrt(1e-5))
    return Problem("large-N N=%d d=30" % n, X, y, "quadratic", _rbf_per_spec(d, dih), 0,
                   optimise_noise=True, swarm=16, iterations=40)


CONFIGS = {1: config1, 2: config2, 3: config3, 5: config5}
