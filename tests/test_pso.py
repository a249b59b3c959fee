"""Host logic of the lockstep PSO driver (no GPU: a numpy evaluator stands in
for the engine's batched call)."""
import numpy as np

from fgpu.pso import LockstepPSO, SwarmConfig


class FakeBatch:
    """ll = -(sum (x - centre)^2); info = 1 where x[0] > fail_above."""

    def __init__(self, centres, owner, fail_above=np.inf):
        self.centres, self.owner, self.fail_above = centres, owner, fail_above
        self.calls = 0

    def __call__(self, positions):
        self.calls += 1
        ll = np.empty(len(positions))
        info = np.zeros(len(positions), dtype=np.int32)
        for k, x in enumerate(positions):
            c = self.centres[self.owner[k]]
            ll[k] = -float(np.sum((np.asarray(x) - c) ** 2))
            if x[0] > self.fail_above:
                info[k] = 7
                ll[k] = np.nan
        return ll, info


def make(nprob=3, S=12, fail_above=np.inf, stall=0):
    boxes = [(np.zeros(2 + a), np.ones(2 + a)) for a in range(nprob)]
    cfg = SwarmConfig(swarm_size=S, iterations=30, stall_iterations=stall, tolerance=1e-12)
    centres = [np.full(2 + a, 0.3 + 0.1 * a) for a in range(nprob)]
    owner = np.repeat(np.arange(nprob), S)
    fake = FakeBatch(centres, owner, fail_above)
    pso = LockstepPSO([(None, lo, hi) for lo, hi in boxes], cfg, seed=3, evaluate=fake)
    return pso, fake, centres


def test_one_batched_call_per_iteration_for_all_swarms():
    pso, fake, _ = make()
    pso.initialise()
    assert fake.calls == 1
    for it in range(5):
        pso.step()
        assert fake.calls == 2 + it


def test_global_best_is_monotone_and_converges():
    pso, fake, centres = make()
    best = pso.run(40)
    for st in pso.states:
        h = np.array(st.history)
        assert np.all(np.diff(h) <= 0)
    for (x, cost), c in zip(best, centres):
        assert cost < 1e-3
        assert np.allclose(x, c, atol=0.05)


def test_failed_particles_are_rerandomised_inside_the_box():
    pso, fake, _ = make(fail_above=0.9)
    pso.initialise()
    for _ in range(6):
        pso.step()
    for st in pso.states:
        assert np.all(np.isfinite(st.cost))     # every particle ended with a successful evaluation
        assert np.all(st.x[:, 0] <= 0.9)
    assert sum(st.failures for st in pso.states) > 0


def test_relative_change_stopping():
    pso, fake, _ = make(stall=3)
    pso.initialise()
    steps = 0
    while not pso.step():
        steps += 1
        assert steps < 500
    assert all(st.stall_count >= 3 for st in pso.states)


class FakeEngine:
    """logL = -sum (x - centre)^2 with its exact gradient (the engine's
    loglik / grad interface)."""

    def __init__(self, centre):
        self.centre = np.asarray(centre, float)
        self.grads = 0

    def loglik(self, x):
        return -float(np.sum((np.asarray(x) - self.centre) ** 2)), 0

    def grad(self, x):
        self.grads += 1
        x = np.asarray(x, float)
        return -float(np.sum((x - self.centre) ** 2)), -2.0 * (x - self.centre), 0


def make_polish(centres, steps, S=6, iterations=3):
    boxes = [(np.zeros(len(c)), np.ones(len(c))) for c in centres]
    cfg = SwarmConfig(swarm_size=S, iterations=iterations, polish_steps=steps)
    owner = np.repeat(np.arange(len(centres)), S)
    fake = FakeBatch([np.asarray(c, float) for c in centres], owner)
    engines = [FakeEngine(c) for c in centres]
    return LockstepPSO([(e, lo, hi) for e, (lo, hi) in zip(engines, boxes)], cfg, seed=5, evaluate=fake), engines


def test_polish_off_leaves_the_trajectory_alone_and_on_only_improves():
    centres = [[0.31, 0.62], [0.2, 0.9, 0.45]]
    plain, e0 = make_polish(centres, steps=0)
    best0 = plain.run()
    assert all(e.grads == 0 for e in e0)          # off: the adjoint is never called
    polished, e1 = make_polish(centres, steps=20)
    best1 = polished.run()
    for s0, s1 in zip(plain.states, polished.states):
        n = len(s0.history)
        assert s1.history[:n] == s0.history        # the swarm's own trajectory is bit-identical
        assert s1.gbest_cost <= s0.gbest_cost
    for (x, cost), c in zip(best1, centres):
        assert cost < 1e-6 and np.allclose(x, c, atol=1e-3)
    assert all(e.grads > 0 for e in e1)


def test_polish_projects_onto_the_box_widened_to_its_start():
    # optimum outside the unit box: the polish ends on the face of the box
    # (widened to contain the swarm's global best, which may be outside it:
    # the reference's swarm has no boundaries), never beyond it
    pso, _ = make_polish([[1.4, 0.5]], steps=40, iterations=2)
    pso.initialise()
    for _ in range(2):
        pso.step()
    x0 = pso.states[0].gbest_x.copy()
    pso.polish()
    x = pso.states[0].gbest_x
    lo, hi = np.minimum(0.0, x0), np.maximum(1.0, x0)
    assert np.all(x >= lo - 1e-15) and np.all(x <= hi + 1e-15)
    assert abs(x[0] - min(1.4, hi[0])) < 1e-3 and abs(x[1] - 0.5) < 1e-3
