"""Autotuner of the batched engine's configuration, per workload shape.

For a batch of problems the tuner times every candidate configuration on a
representative sample of the batch, keeps the fastest and caches the choice
on disk under the batch's shape key, so that another swarm (or another
process) of the same shape reuses it without timing again.

Candidates -- each evaluates the same likelihood to the parity tolerance;
they differ in speed only, and which is fastest depends on the shape:

* ``tcgen05/tc``:   split-integer tensor-core trailing update (128-wide
  panels) and the tensor-core exact-distance kernel-matrix build;
* ``tcgen05/fp64``: the same update with the FP64 dot-product build (cheaper
  per entry for a few features: no digit planes, no TMEM drains);
* ``fp64/fp64``:    the all-FP64 engine (64-wide panels, FP64 ``mma.sync``
  update), which has the least fixed cost per panel step.

Shape key: device name and SM count, the largest N rounded up to a power of
two, the largest feature count d, the batch size rounded up to a power of
two, and the kernel's leaf types.  The cache file is ``$FGPU_TUNE_CACHE``, or
``~/.cache/fgpu/tune.json``.

The timer is a parameter: ``gpu_timer`` builds engines under a candidate and
times replays of a batch plan on the device; tests pass a fake.
"""
from __future__ import annotations

import json
import os
import time
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Config:
    trailing: str = "tcgen05"   # "tcgen05" | "fp64"
    build: str = "tc"           # "tc" | "fp64"

    @property
    def name(self):
        return f"{self.trailing}/{self.build}"

    @staticmethod
    def from_name(name):
        t, b = name.split("/")
        return Config(t, b)


DEFAULT = Config()
CANDIDATES = (Config("tcgen05", "tc"), Config("tcgen05", "fp64"), Config("fp64", "fp64"))


@dataclass
class Workload:
    """One problem of a batch: the data an engine is created from, and how
    many particles of it the batch holds."""
    X: np.ndarray
    y: np.ndarray
    mu: np.ndarray
    kspec: list
    likelihood: int
    noise: float
    optimise_noise: bool
    particles: int = 1

    @property
    def N(self):
        return int(np.asarray(self.X).shape[0])

    @property
    def d(self):
        return int(np.asarray(self.X).shape[1])


def _pow2(n):
    return 1 << max(0, int(n - 1).bit_length())


def shape_key(workloads, device="cpu", sms=0):
    from .kernel_spec import parse_kspec
    nmax = max(w.N for w in workloads)
    dmax = max(w.d for w in workloads)
    batch = sum(w.particles for w in workloads)
    leaves = sorted({n[1] for w in workloads for n in parse_kspec(w.kspec) if n[0] == "leaf"})
    return (f"{device}|sms{sms}|N{_pow2(nmax)}|d{dmax}|B{_pow2(batch)}|lik"
            f"{sorted({w.likelihood for w in workloads})}|leaves{leaves}")


class TuneCache:
    """{shape key: {"choice": name, "ms": {name: milliseconds}}} on disk."""

    def __init__(self, path=None):
        self.path = path or os.environ.get("FGPU_TUNE_CACHE") or os.path.join(
            os.path.expanduser("~"), ".cache", "fgpu", "tune.json")
        self.data = {}
        try:
            with open(self.path) as f:
                self.data = json.load(f)
        except (OSError, ValueError):
            self.data = {}

    def get(self, key):
        e = self.data.get(key)
        return Config.from_name(e["choice"]) if e else None

    def put(self, key, choice, ms):
        self.data[key] = {"choice": choice.name, "ms": ms}
        os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
        # a temporary file of this process's own, renamed over the cache in
        # one step: ranks of one job that tune at the same time never share
        # the temporary (one's rename would leave the other nothing to
        # rename) and a reader sees one whole file or the other
        tmp = f"{self.path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(self.data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def sample_batch(workloads, max_problems=8):
    """A representative sample of the batch: the largest problems first (the
    factorisation's N^3 dominates), each with its particle count, up to
    ``max_problems`` evaluations."""
    order = sorted(range(len(workloads)), key=lambda a: -workloads[a].N)
    out, left = [], max_problems
    for a in order:
        if left <= 0:
            break
        k = min(workloads[a].particles, left)
        w = workloads[a]
        out.append(Workload(w.X, w.y, w.mu, w.kspec, w.likelihood, w.noise, w.optimise_noise, k))
        left -= k
    return out


def tune(workloads, timer=None, cache=None, candidates=CANDIDATES, device="cpu", sms=0, retune=False):
    """Pick the fastest candidate for this batch.  Returns (Config, {name: ms},
    from_cache)."""
    key = shape_key(workloads, device, sms)
    cache = cache if cache is not None else TuneCache()
    if not retune:
        hit = cache.get(key)
        if hit is not None:
            return hit, cache.data[key].get("ms", {}), True
    timer = timer or gpu_timer
    sample = sample_batch(workloads)
    ms = {}
    for c in candidates:
        try:
            ms[c.name] = 1e3 * float(timer(c, sample))
        except Exception:   # a candidate that cannot run this shape is not chosen
            ms[c.name] = float("inf")
    best = min(candidates, key=lambda c: ms[c.name])
    if not np.isfinite(ms[best.name]):
        best = DEFAULT
    cache.put(key, best, ms)
    return best, ms, False


class use:
    """Context manager: engines created inside it get configuration ``cfg``."""

    def __init__(self, cfg):
        self.cfg = cfg

    def __enter__(self):
        from .gpr import set_build_mode, set_trailing_update
        self.prev = (set_trailing_update(self.cfg.trailing), set_build_mode(self.cfg.build))
        return self

    def __exit__(self, *a):
        from .gpr import set_build_mode, set_trailing_update
        set_trailing_update(self.prev[0])
        set_build_mode(self.prev[1])


def gpu_timer(cfg, sample, reps=3, seed=0):
    """Seconds per replay of a batch plan over ``sample`` under ``cfg``
    (host theta in, ll / info out; one warm-up replay)."""
    from .gpr import Engine, Plan
    with use(cfg):
        engines = [Engine(w.X, w.y, w.mu, w.kspec, w.likelihood, w.noise, w.optimise_noise) for w in sample]
    flat = [e for e, w in zip(engines, sample) for _ in range(w.particles)]
    rng = np.random.default_rng(seed)
    th = [rng.uniform(0.0, 1.0, size=e.ntheta) for e in flat]
    for e, t in zip(flat, th):
        if e.optimise_noise:
            t[-1] = 1e-8
    plan = Plan(flat)
    plan.run(th)
    t0 = time.perf_counter()
    for _ in range(reps):
        plan.run(th)
    dt = (time.perf_counter() - t0) / reps
    plan.close()
    for e in engines:
        e.close()
    return dt


def device_identity():
    """(device name, SM count) of the current CUDA device, for shape keys."""
    try:
        import torch
        p = torch.cuda.get_device_properties(torch.cuda.current_device())
        return p.name.replace(" ", "_"), int(p.multi_processor_count)
    except Exception:
        return "unknown", 0
