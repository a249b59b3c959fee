"""The adjoint as a torch.autograd.Function (test harness) and the
off-by-default gradient polish of the swarm's global best, on the GPU."""
import numpy as np
import pytest

from oracle import gpr_oracle as O

pytestmark = pytest.mark.gpu


def _small_problem(seed=2, n=150):
    rng = np.random.default_rng(seed)
    X = rng.normal(2.0, 0.3, size=(n, 4))
    X[:, -1] = rng.uniform(-np.pi, np.pi, size=n)
    y = np.cos(X[:, 0]) + 0.2 * np.sin(X[:, -1]) + 1e-3 * rng.normal(size=n)
    ks = [O.RBF, 3, 1, 2, 3, O.PERIODIC, 1, 4, O.SUM]
    return X, y, O.mean_vector("constant", X, y), ks


@pytest.mark.parametrize("optimise_noise", [False, True])
def test_autograd_function_against_gradcheck_and_the_oracle(optimise_noise, lib):
    torch = pytest.importorskip("torch")
    from autograd_fgpu import loglik
    from fgpu import Engine
    X, y, mu, ks = _small_problem()
    e = Engine(X, y, mu, ks, 0, 1e-6, optimise_noise)
    th0 = np.array([0.3, 0.6, 0.2, 0.5] + ([1e-4] if optimise_noise else []))
    th = torch.tensor(th0, dtype=torch.float64, requires_grad=True)
    ll = loglik(th, e)
    ll.backward()
    _, g_ref, info = O.loglik_grad(ks, th0, X, y, mu, 0, 1e-6, optimise_noise)
    assert info == 0
    assert np.allclose(th.grad.numpy(), g_ref, rtol=1e-6, atol=1e-8 * np.max(np.abs(g_ref)))
    # torch's own finite-difference check of the backward against the forward,
    # over the kernel parameters (the noise, 1e-4, would not survive an
    # absolute step of eps; its derivative is checked against the oracle
    # above); eps = 1e-4: with 1e-6 the differences are dominated by the
    # forward's rounding (~1e-12 of logL at this conditioning)
    nk = 4
    rest = torch.tensor(th0[nk:], dtype=torch.float64)
    assert torch.autograd.gradcheck(lambda t: loglik(torch.cat([t, rest]), e),
                                    (torch.tensor(th0[:nk], dtype=torch.float64, requires_grad=True),),
                                    eps=1e-4, atol=1e-4, rtol=1e-4)


def test_polish_of_the_large_n_swarm(lib):
    """Large-N set (N=10000, d=30, quadratic mean, optimised noise), swarm of
    16: with the polish off the swarm's trajectory is what it is; with it on
    the same trajectory (bit for bit) is followed by accepted gradient steps,
    and the final logL is no lower."""
    from fgpu import Engine, synth
    from fgpu.pso import LockstepPSO, SwarmConfig
    p = synth.config5()
    mu = O.mean_vector(p.mean, p.X, p.y)
    e = Engine(p.X, p.y, mu, p.kspec, p.likelihood, p.noise, p.optimise_noise)
    nk = e.ntheta - 1
    lo = np.r_[np.full(nk, p.theta_lo), 1e-12]
    hi = np.r_[np.full(nk, p.theta_hi), 1e-6]
    runs = []
    for steps in (0, 4):
        cfg = SwarmConfig(swarm_size=16, iterations=10, polish_steps=steps)
        pso = LockstepPSO([(e, lo, hi)], cfg, seed=5)
        (x, cost), = pso.run()
        runs.append((pso.states[0].history, x, cost, getattr(pso, "polish_accepted", [[]])[0]))
        del pso
    (h0, x0, c0, _), (h1, x1, c1, acc) = runs
    assert h1[:len(h0)] == h0
    assert c1 <= c0 and np.isfinite(c1)
    ll1, info = e.loglik(x1)
    assert info == 0 and abs(-ll1 - c1) <= 1e-12 * abs(c1)
    print(f"large-N polish: -logL {c0:.10g} -> {c1:.10g} ({len(acc)} accepted steps)")
