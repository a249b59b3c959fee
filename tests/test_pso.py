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
