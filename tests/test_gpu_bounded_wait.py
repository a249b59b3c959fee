"""A bounded wait that gives up is an error status, not a hang or a fault.

Every mbarrier wait in the tensor-core kernels polls at most 2^22 times; on
giving up the kernel sets a status word, which the host reports as
FGPU_ETIMEOUT.  fgpu_diag_wait runs that same wait helper on a barrier that
nothing arrives on, with a few polls and nothing asynchronous in flight, so
the give-up path is exercised without faulting or hanging the GPU.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FGPU_ETIMEOUT = -5


def test_wait_that_nobody_completes_gives_up_with_a_status(lib):
    assert lib.fgpu_diag_wait(64, 0) == FGPU_ETIMEOUT
    assert b"bounded wait" in lib.fgpu_last_error()


def test_completed_wait_passes_and_the_device_stays_usable(lib):
    from fgpu import Engine
    from oracle import gpr_oracle as O
    assert lib.fgpu_diag_wait(64, 0) == FGPU_ETIMEOUT
    assert lib.fgpu_diag_wait(64, 1) == 0
    rng = np.random.default_rng(8)
    X = rng.normal(2.0, 0.3, size=(200, 3))
    y = np.sin(X[:, 0]) + 1e-3 * rng.normal(size=200)
    ks = [O.RBF, 3, 1, 2, 3]
    mu = O.mean_vector("constant", X, y)
    e = Engine(X, y, mu, ks, 0, 1e-6, False)
    th = np.array([0.3, 0.5, 0.7])
    ll, info = e.loglik(th)
    ref, rinfo = O.loglik(ks, th, X, y, mu, 0, 1e-6, False)
    assert info == rinfo == 0 and abs(ll - ref) <= 1e-9 * abs(ref)


def test_diag_wait_rejects_bad_arguments(lib):
    assert lib.fgpu_diag_wait(0, 0) == -1
    assert lib.fgpu_diag_wait(64, 2) == -1
