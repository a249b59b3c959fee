"""Host-side mirror of FEREBUS-v7's GPR cost-function interface over the C-ABI.

``GaussianProcessRegressor`` follows the reference's ``Optimisable`` contract
(src/model/gpr/gpr.f90:52-121): ``set_params``/``get_params``/``nparams``,
``search_min``/``search_max`` and ``cost_function(param) -> IterResult`` with
cost = -logL and ``success = (info == 0)`` (src/optimiser/iter_result.f90:92-101).
The numeric work behind ``log_likelihood`` runs in libfgpu.so; nothing here
evaluates a kernel or a factorisation on the CPU.

The engine context is created once per training set (the reference
re-initialises S GPR objects every PSO iteration, src/optimiser/pso/pso.f90:411-414,
so per-particle objects share one ``Engine``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .kernel_spec import CONSTANT, build_kspec, parse_kspec, nparams as spec_nparams

MARGINAL, CONCENTRATED = 0, 1
LIKELIHOODS = {"marginal": MARGINAL, "concentrated": CONCENTRATED}


def _dp(a):
    return a.ctypes.data_as(_lib.c_double_p)


class Engine:
    """One training set resident on the GPU (an ``fgpu_ctx``)."""

    def __init__(self, X, y, mu, kspec, likelihood=MARGINAL, noise=1e-10, optimise_noise=False):
        self.lib = _lib.load()
        X = np.asarray(X, dtype=np.float64)
        if X.ndim != 2:
            raise ValueError("X must be (N, d)")
        self.N, self.d = X.shape
        self._X = np.asfortranarray(X)               # column-major, as Fortran stores X(N, d)
        self._y = np.ascontiguousarray(y, dtype=np.float64)
        self._mu = None if mu is None else np.ascontiguousarray(mu, dtype=np.float64)
        if self._y.shape != (self.N,) or (self._mu is not None and self._mu.shape != (self.N,)):
            raise ValueError("y / mu must have length N")
        self.kspec = [int(v) for v in kspec]
        self.likelihood = int(likelihood)
        self.noise = float(noise)
        self.optimise_noise = bool(optimise_noise)
        ks = (C.c_int * len(self.kspec))(*self.kspec)
        h = C.c_void_p()
        mu_p = _dp(self._mu) if self._mu is not None else None
        _lib.check(self.lib.fgpu_create(C.byref(h), self.N, self.d, _dp(self._X), _dp(self._y), mu_p, ks,
                                        len(self.kspec), self.likelihood, self.noise,
                                        1 if self.optimise_noise else 0))
        self.handle = h
        self.ntheta = self.lib.fgpu_nparams(h)

    def loglik(self, theta, want_alpha=False):
        """Returns ``(ll, info)`` or ``(ll, info, alpha)``."""
        th = np.ascontiguousarray(theta, dtype=np.float64)
        ll, info = C.c_double(), C.c_int()
        alpha = np.empty(self.N) if want_alpha else None
        _lib.check(self.lib.fgpu_loglik(self.handle, _dp(th), th.size, C.byref(ll), C.byref(info),
                                        _dp(alpha) if want_alpha else None))
        if want_alpha:
            return ll.value, info.value, alpha
        return ll.value, info.value

    def grad(self, theta):
        """Returns ``(ll, dll_dtheta, info)`` from the FP64 adjoint."""
        th = np.ascontiguousarray(theta, dtype=np.float64)
        ll, info = C.c_double(), C.c_int()
        g = np.empty(self.ntheta)
        _lib.check(self.lib.fgpu_grad(self.handle, _dp(th), th.size, C.byref(ll), _dp(g), C.byref(info)))
        return ll.value, g, info.value

    def clone(self):
        """A new context on the same training set, created under the current
        process-wide trailing-update and build modes."""
        return Engine(self._X, self._y, self._mu, self.kspec, self.likelihood, self.noise, self.optimise_noise)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fgpu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """A fixed batch of problems (``fgpu_plan``): one graph replay per call."""

    def __init__(self, engines, ldtheta=None):
        self.lib = _lib.load()
        self.engines = list(engines)
        self.nprob = len(self.engines)
        self.ldtheta = int(ldtheta or max(e.ntheta for e in self.engines))
        arr = (C.c_void_p * self.nprob)(*[e.handle.value for e in self.engines])
        h = C.c_void_p()
        _lib.check(self.lib.fgpu_plan_create(C.byref(h), arr, self.nprob, self.ldtheta))
        self.handle = h

    def run(self, thetas):
        """thetas: (nprob, ldtheta) host array -> (ll, info)."""
        th = np.zeros((self.nprob, self.ldtheta))
        for i, t in enumerate(thetas):
            t = np.asarray(t, dtype=np.float64)
            th[i, :t.size] = t
        ll = np.empty(self.nprob)
        info = np.empty(self.nprob, dtype=np.int32)
        _lib.check(self.lib.fgpu_plan_run(self.handle, _dp(th), _dp(ll),
                                          info.ctypes.data_as(_lib.c_int_p)))
        return ll, info

    def run_device(self, theta_ptr, ll_ptr, info_ptr, stream_ptr=None):
        """Device pointers (ints) in and out; enqueued on ``stream_ptr``."""
        _lib.check(self.lib.fgpu_plan_run_device(self.handle, C.c_void_p(theta_ptr), C.c_void_p(ll_ptr),
                                                 C.c_void_p(info_ptr), C.c_void_p(stream_ptr or 0)))

    def launches(self):
        return int(self.lib.fgpu_last_launch_count())

    def waves(self):
        """(number of waves, bytes of the shared workspace arena)."""
        nw, ab = C.c_int(), C.c_longlong()
        _lib.check(self.lib.fgpu_plan_waves(self.handle, C.byref(nw), C.byref(ab)))
        return nw.value, ab.value

    def set_profiling(self, enable=True):
        """True: event nodes around every launch; "update": around the
        trailing-update launches only; False: off."""
        mode = 2 if enable == "update" else (1 if enable else 0)
        _lib.check(self.lib.fgpu_plan_set_profiling(self.handle, mode))

    STAGES = ("build", "potf2", "trsm", "update", "finalize", "panel_prep", "split", "border", "coupling")

    def stage_times(self):
        """{stage: (ms during the last replay, launches)}."""
        ms = np.zeros(len(self.STAGES))  # FGPU_NSTAGES entries
        cnt = np.zeros(len(self.STAGES), dtype=np.int32)
        _lib.check(self.lib.fgpu_plan_stage_times(self.handle, _dp(ms), cnt.ctypes.data_as(_lib.c_int_p)))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.STAGES)}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fgpu_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_trailing_update(mode):
    """Trailing-update arithmetic for engines created afterwards: "tcgen05"
    (default, exact split-integer products on the tensor cores) or "fp64".
    Returns the previous mode name."""
    lib = _lib.load()
    code = {"fp64": 0, "tcgen05": 1}[mode]
    prev = _lib.check(lib.fgpu_set_trailing_update(code))
    return {0: "fp64", 1: "tcgen05"}[prev]


def plan_partition(nbytes, budget):
    """The wave partition a plan applies to problems with these workspace
    sizes under ``budget`` bytes (host-only): returns (wave of each problem,
    number of waves)."""
    lib = _lib.load()
    n = len(nbytes)
    b = (C.c_longlong * n)(*[int(v) for v in nbytes])
    w = (C.c_int * n)()
    nw = C.c_int()
    _lib.check(lib.fgpu_plan_partition(b, n, int(budget), w, C.byref(nw)))
    return list(w), nw.value


def set_build_mode(mode):
    """Kernel-matrix build for engines created afterwards: "tc" (default,
    exact distances on the tensor cores where the kernel allows) or "fp64"
    (the FP64 dot-product form).  Returns the previous mode name."""
    lib = _lib.load()
    prev = _lib.check(lib.fgpu_set_build_mode({"fp64": 0, "tc": 1}[mode]))
    return {0: "fp64", 1: "tc"}[prev]


def loglik_batch(engines, thetas):
    """``fgpu_loglik_batch``: a ragged list of (engine, theta) problems."""
    lib = _lib.load()
    n = len(engines)
    arr = (C.c_void_p * n)(*[e.handle.value for e in engines])
    keep = [np.ascontiguousarray(t, dtype=np.float64) for t in thetas]
    tp = (_lib.c_double_p * n)(*[_dp(t) for t in keep])
    ll = np.empty(n)
    info = np.empty(n, dtype=np.int32)
    _lib.check(lib.fgpu_loglik_batch(arr, n, tp, _dp(ll), info.ctypes.data_as(_lib.c_int_p)))
    return ll, info


@dataclass
class IterResult:
    """src/optimiser/iter_result.f90:92-101: success = (info == 0)."""
    param: np.ndarray
    cost: float
    info: int

    @property
    def success(self):
        return self.info == 0


def mean_vector(kind, X, y):
    """Host mean functions (computed once per data set, src/mean/*.f90): zero,
    constant = mean(y), linear / quadratic least squares anchored at argmin y
    (src/mean/least_squares.f90:54-93; normal equations solved by Cholesky as
    dposv('L') does)."""
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n, d = X.shape
    if kind == "zero":
        return np.zeros(n)
    if kind == "constant":
        return np.full(n, float(np.sum(y)) / n)
    if kind in ("linear", "quadratic"):
        imin = int(np.argmin(y))
        xmin, ymin = X[imin].copy(), y[imin]
        a = X - xmin
        if kind == "quadratic":
            a = a * a
        L = np.linalg.cholesky(a.T @ a)
        beta = np.linalg.solve(L.T, np.linalg.solve(L, a.T @ (y - ymin)))
        return a @ beta + ymin
    raise ValueError(f"unknown mean {kind!r}")


class GaussianProcessRegressor:
    """Mirror of ``GaussianProcessRegressor`` (src/model/gpr/gpr.f90:98-121).

    ``kernel`` is the model's kernel expression (e.g. ``"k1*k2"``) and
    ``kernels`` the ``[kernels.*]`` tables (``type``, ``active_dimensions``).
    ``search_min``/``search_max`` default to the reference's 0 / 1
    (src/config/optimiser/optimiser.f90:34-38); the noise box is [1e-12, 1e-6]
    (gpr.f90:221-245).
    """

    def __init__(self, X, y, kernel="k1", kernels=None, mean="constant", likelihood="marginal",
                 noise=1e-10, optimise_noise=False, search_min=0.0, search_max=1.0, engine=None):
        X = np.asarray(X, dtype=np.float64)
        self.X, self.y = X, np.asarray(y, dtype=np.float64)
        kernels = kernels or {"k1": {"type": "rbf"}}
        self.kspec, consts = build_kspec(kernel, kernels, X.shape[1])
        self.likelihood = LIKELIHOODS[likelihood] if isinstance(likelihood, str) else int(likelihood)
        self.nugget = float(noise)
        self.optimise_nugget = bool(optimise_noise)
        self.cached_mean = mean_vector(mean, X, self.y)            # gpr.f90:168-171
        self.engine = engine or Engine(X, self.y, self.cached_mean, self.kspec, self.likelihood, noise,
                                       optimise_noise)
        self._search = (float(search_min), float(search_max))
        # a number in the expression is a constant kernel whose parameter is
        # its value, starting at that number (visit_numop,
        # src/interpreter/ast.f90:257-271); the other parameters start at 0
        # here (the swarm sets every parameter before the first evaluation)
        self.params = np.zeros(self.nparams())
        off, k = 0, 0
        for node in parse_kspec(self.kspec):
            if node[0] != "leaf":
                continue
            if node[1] == CONSTANT:
                self.params[off] = float(consts[k])
                k += 1
                off += 1
            else:
                off += len(node[2])

    def nparams(self):
        return spec_nparams(self.kspec) + (1 if self.optimise_nugget else 0)

    def set_params(self, params):
        """gpr.f90:191-202 (the transforms themselves happen on the device)."""
        params = np.asarray(params, dtype=np.float64)
        if params.size != self.nparams():
            raise ValueError(f"expected {self.nparams()} parameters")
        self.params = params.copy()
        if self.optimise_nugget:
            self.nugget = float(params[-1])

    def get_params(self):
        return self.params.copy()

    def search_min(self):
        m = np.full(self.nparams(), self._search[0])
        if self.optimise_nugget:
            m[-1] = 1e-12
        return m

    def search_max(self):
        m = np.full(self.nparams(), self._search[1])
        if self.optimise_nugget:
            m[-1] = 1e-6
        return m

    def log_likelihood(self):
        """gpr.f90:291-307 -> (ll, info)."""
        return self.engine.loglik(self.params)

    def cost_function(self, param):
        """negative_log_likelihood (gpr.f90:258-289)."""
        self.set_params(param)
        ll, info = self.log_likelihood()
        return IterResult(np.asarray(param, dtype=np.float64).copy(), -ll, info)

    def weights(self):
        """alpha = K^-1 (y - mu), the model file's [weights] (likelihood.f90:255-264)."""
        ll, info, alpha = self.engine.loglik(self.params, want_alpha=True)
        return alpha, info
