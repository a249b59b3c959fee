"""Lockstep particle-swarm driver over the batched engine.

Host-side mirror of FEREBUS-v7's global swarm updater
(src/optimiser/pso/pso.f90:382-472, init_pso 250-368) in which every
particle of an iteration -- and, for a multi-atom run, every particle of every
atom's swarm -- is evaluated in ONE batched engine call (``Plan``), instead of
one OpenMP thread per particle calling the likelihood (pso.f90:419-452).

Per iteration and particle i (pso.f90:419-452):
    v_i <- w v_i + c1 r1 (pbest_i - x_i) + c2 r2 (gbest - x_i),  x_i <- x_i + v_i
then the swarm's costs are evaluated together; a particle whose Cholesky
fails (info != 0) is re-randomised in its search box and re-evaluated
(get_cost, src/optimiser/pso/particle.f90:149-162) in follow-up batches; then
personal bests, then the global best in particle order (pso.f90:454-459,
"<=" comparisons).  The initial swarm is evaluated once without retries
(init_particle, particle.f90:53-100); a failed initial particle starts with
cost +inf.  Stopping: a fixed iteration count (optimiser_type.f90:118-133) or
the relative-change criterion (pso.f90:619-636).

The forced swarm updater (pso.f90:485-558) updates the global best inside the
particle loop, so its trajectory is inherently sequential; it is not offered
here.  Random numbers come from numpy's PCG64, not the reference's RNG, so
trajectories match the reference in distribution, not bit for bit.

Gradient polish (``SwarmConfig.polish_steps > 0``; off by default, and then
nothing below runs): after the last iteration each swarm's global best is
refined by projected gradient ascent on logL with the engine's FP64 adjoint
(``fgpu_grad``), in box-normalised coordinates u = (theta - lo) / (hi - lo)
so that the linear noise parameter (box [1e-12, 1e-6]) and the kernel
parameters move on the same scale.  Each step tries a move of at most
``polish_move`` of the box along the gradient, halves it until logL improves
(at most ``polish_halvings`` times) and keeps only improving moves, so the
polished cost is never above the swarm's.  Moves are projected onto the
search box widened to contain the starting point: the reference's swarm has
no search boundaries (pso.f90:431, "TODO: Implement search boundaries") and
its global best may lie outside the box, and the polish goes no further out.  The reference has no gradient
(negative_log_likelihood, src/model/gpr/gpr.f90:258-289, ignores its
``gradient`` flag); the polish starts from the global best the reference's
serial update keeps (pso.f90:454-459) and leaves the swarm's trajectory
untouched.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .gpr import Plan


@dataclass
class SwarmConfig:
    """[optimiser.pso] of the reference's TOML (src/config/optimiser/pso/pso.f90)."""
    swarm_size: int = 50
    iterations: int = 1000
    inertia_weight: float = 0.729
    cognitive_learning_rate: float = 1.494
    social_learning_rate: float = 1.494
    stall_iterations: int = 0        # 0: no relative-change stopping
    tolerance: float = 1e-8
    max_retries: int = 64            # bound on re-randomisations per particle per iteration
    polish_steps: int = 0            # gradient-polish steps of each global best (0: off)
    polish_move: float = 0.05        # largest first move per step, as a fraction of the box
    polish_halvings: int = 10


@dataclass
class SwarmState:
    x: np.ndarray
    v: np.ndarray
    cost: np.ndarray
    pbest_x: np.ndarray
    pbest_cost: np.ndarray
    gbest_x: np.ndarray
    gbest_cost: float
    lo: np.ndarray
    hi: np.ndarray
    history: list = field(default_factory=list)
    stall_count: int = 0
    stall_cost: float = np.inf
    evaluations: int = 0
    failures: int = 0


class LockstepPSO:
    """One PSO per problem (atom / property); all swarms advance together.

    ``problems`` is a list of ``(engine, search_min, search_max)``; each
    engine is an ``fgpu.Engine`` (one training set).  Cost = -logL.

    Random numbers: one generator seeded by ``seed`` for all swarms, or, with
    ``seeds`` (one per problem), a generator per swarm, so that a swarm's
    trajectory does not depend on which other swarms share the batch (what
    ``fgpu.partition.train_sharded`` relies on to give the same result on
    any number of ranks).
    """

    def __init__(self, problems, config: SwarmConfig, seed=17, evaluate=None, tune=False, seeds=None):
        self.cfg = config
        self.rng = np.random.default_rng(seed)
        if seeds is not None and len(seeds) != len(problems):
            raise ValueError("seeds: one per problem")
        self.rngs = ([np.random.default_rng(x) for x in seeds] if seeds is not None
                     else [self.rng] * len(problems))
        self.engines = [p[0] for p in problems]
        self.boxes = [(np.asarray(p[1], float), np.asarray(p[2], float)) for p in problems]
        self.ntheta = [len(b[0]) for b in self.boxes]
        S = config.swarm_size
        self.owner = np.repeat(np.arange(len(problems)), S)
        self.tuned = None
        if evaluate is None:
            if tune:
                # the engine configuration fastest for this batch's shape
                # (fgpu.autotune; timed once per shape, then cached on disk)
                from . import autotune
                wl = [autotune.Workload(e._X, e._y, e._mu, e.kspec, e.likelihood, e.noise, e.optimise_noise, S)
                      for e in self.engines]
                dev, sms = autotune.device_identity()
                self.tuned, self.tune_ms, _ = autotune.tune(wl, device=dev, sms=sms)
                with autotune.use(self.tuned):
                    self.engines = [e.clone() for e in self.engines]
            plan = Plan([e for e in self.engines for _ in range(S)], ldtheta=max(self.ntheta))
            evaluate = plan.run
            self.plan = plan
        self.evaluate_batch = evaluate   # list of positions -> (ll, info)
        self.states = []

    # -- batched cost evaluation with the reference's retry rule -------------
    def _evaluate(self, positions, retry):
        """positions: list over all particles (each its problem's ntheta).
        Returns costs (+inf for particles that failed and were not retried)."""
        S = self.cfg.swarm_size
        ll, info = self.evaluate_batch(positions)
        ll, info = np.asarray(ll, float), np.asarray(info)
        cost = -ll
        bad = np.nonzero(info != 0)[0]
        tries = 0
        while retry and bad.size and tries < self.cfg.max_retries:
            tries += 1
            for k in bad:
                a = self.owner[k]
                lo, hi = self.boxes[a]
                st = self.states[a]
                i = k - a * S
                delta = hi - lo
                st.x[i] = self.rngs[a].uniform(lo, hi)
                st.v[i] = self.rngs[a].uniform(-delta, delta)
                positions[k] = st.x[i]
                st.failures += 1
            ll, info2 = self.evaluate_batch(positions)
            mask = np.isin(np.arange(len(cost)), bad)
            cost = np.where(mask, -np.asarray(ll, float), cost)
            info = np.where(mask, np.asarray(info2), 0)
            bad = np.nonzero(info != 0)[0]
        for k in bad:
            cost[k] = np.inf
        for a, st in enumerate(self.states):
            st.evaluations += S
        return cost

    def _positions(self):
        return [st.x[i] for st in self.states for i in range(self.cfg.swarm_size)]

    def initialise(self):
        """init_pso: uniform positions in the box, velocities in +-(max - min)."""
        S = self.cfg.swarm_size
        self.states = []
        for a, ((lo, hi), n) in enumerate(zip(self.boxes, self.ntheta)):
            delta = hi - lo
            x = self.rngs[a].uniform(lo, hi, size=(S, n))
            v = self.rngs[a].uniform(-delta, delta, size=(S, n))
            self.states.append(SwarmState(x=x, v=v, cost=np.full(S, np.inf), pbest_x=x.copy(),
                                          pbest_cost=np.full(S, np.inf), gbest_x=x[0].copy(),
                                          gbest_cost=np.inf, lo=lo, hi=hi))
        cost = self._evaluate(self._positions(), retry=False)
        for a, st in enumerate(self.states):
            c = cost[a * S:(a + 1) * S]
            st.cost[:] = c
            st.pbest_cost[:] = c
            st.pbest_x[:] = st.x
            for i in range(S):
                if c[i] <= st.gbest_cost:
                    st.gbest_cost = c[i]
                    st.gbest_x = st.x[i].copy()
            st.history.append(st.gbest_cost)

    def step(self):
        """One global_swarm_update for every swarm, one batched evaluation."""
        cfg, S = self.cfg, self.cfg.swarm_size
        for a, st in enumerate(self.states):
            n = st.x.shape[1]
            r1 = self.rngs[a].random((S, n))
            r2 = self.rngs[a].random((S, n))
            st.v = (cfg.inertia_weight * st.v + cfg.cognitive_learning_rate * r1 * (st.pbest_x - st.x)
                    + cfg.social_learning_rate * r2 * (st.gbest_x - st.x))
            st.x = st.x + st.v
        cost = self._evaluate(self._positions(), retry=True)
        done = []
        for a, st in enumerate(self.states):
            c = cost[a * S:(a + 1) * S]
            st.cost[:] = c
            better = c <= st.pbest_cost
            st.pbest_x[better] = st.x[better]
            st.pbest_cost[better] = c[better]
            for i in range(S):
                if c[i] <= st.gbest_cost:
                    st.gbest_cost = c[i]
                    st.gbest_x = st.x[i].copy()
            st.history.append(st.gbest_cost)
            done.append(self._stop(st))
        return all(done)

    def _stop(self, st):
        """Relative-change stopping criterion (pso.f90:619-636)."""
        if self.cfg.stall_iterations <= 0:
            return False
        # the first check divides by the initial infinite stall cost: NaN, which
        # compares false in the reference, i.e. a reset
        if (np.isfinite(st.stall_cost) and st.stall_cost != 0
                and abs((st.gbest_cost - st.stall_cost) / st.stall_cost) <= self.cfg.tolerance):
            st.stall_count += 1
        else:
            st.stall_count = 0
            st.stall_cost = st.gbest_cost
        return st.stall_count >= self.cfg.stall_iterations

    def run(self, iterations=None):
        self.initialise()
        for _ in range(iterations if iterations is not None else self.cfg.iterations):
            if self.step():
                break
        if self.cfg.polish_steps > 0:
            self.polish()
        return [(st.gbest_x, st.gbest_cost) for st in self.states]

    def polish(self, steps=None):
        """Projected gradient ascent on logL from each swarm's global best
        (see the module docstring); updates gbest_x / gbest_cost only where
        logL improves.  Returns per swarm the list of accepted costs."""
        steps = self.cfg.polish_steps if steps is None else steps
        out = []
        for a, st in enumerate(self.states):
            eng = self.engines[a]
            x, cost = st.gbest_x.copy(), st.gbest_cost
            width = np.where(st.hi > st.lo, st.hi - st.lo, 1.0)
            lo, hi = np.minimum(st.lo, x), np.maximum(st.hi, x)
            accepted = []
            if not np.isfinite(cost):
                out.append(accepted)
                continue
            for _ in range(steps):
                ll, g, info = eng.grad(x)
                if info != 0 or not np.all(np.isfinite(g)):
                    break
                gu = g * width                      # d logL / du
                norm = float(np.max(np.abs(gu)))
                if norm == 0.0:
                    break
                t = self.cfg.polish_move / norm
                moved = False
                for _h in range(self.cfg.polish_halvings + 1):
                    xn = np.clip(x + t * gu * width, lo, hi)
                    lln, infon = eng.loglik(xn)
                    if infon == 0 and np.isfinite(lln) and -lln < cost:
                        x, cost, moved = xn, -lln, True
                        break
                    t *= 0.5
                if not moved:
                    break
                accepted.append(cost)
            st.gbest_x, st.gbest_cost = x, cost
            st.history.append(cost)
            out.append(accepted)
        self.polish_accepted = out
        return out
