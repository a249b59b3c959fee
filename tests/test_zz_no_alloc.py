"""fgpu_loglik_noalloc: the evaluation path for callers that cannot allocate
device memory (an OpenACC host whose device memory belongs to the OpenACC
runtime, a pool that forbids side allocations, a thread running while a
global-mode stream capture is active).  Its intermediates live in a fixed
static device array, so it takes device pointers in and out and rejects
N > FGPU_NOALLOC_MAX_N.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import gpr_oracle as O

NOALLOC_MAX_N = 1024


def _problem(n, d, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(2.0, 0.3, size=(n, d))
    X[:, -1] = rng.uniform(-np.pi, np.pi, size=n)
    y = np.cos(X[:, 0]) + 0.2 * np.sin(X[:, -1]) + 1e-3 * rng.normal(size=n)
    ks = [O.RBF, d - 1] + list(range(1, d)) + [O.PERIODIC, 1, d, O.SUM]
    mu = O.mean_vector("constant", X, y)
    return X, y, mu, ks


def _call_noalloc(lib, torch, X, y, mu, ks, lik, noise, optimise_noise, theta, stream):
    n, d = X.shape
    Xd = torch.tensor(np.asfortranarray(X).ravel(order="F"), dtype=torch.float64, device="cuda")
    yd = torch.tensor(y, dtype=torch.float64, device="cuda")
    mud = torch.tensor(mu, dtype=torch.float64, device="cuda")
    thd = torch.tensor(theta, dtype=torch.float64, device="cuda")
    lld = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    infod = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    ksa = (C.c_int * len(ks))(*ks)
    rc = lib.fgpu_loglik_noalloc(n, d, C.c_void_p(Xd.data_ptr()), C.c_void_p(yd.data_ptr()),
                                 C.c_void_p(mud.data_ptr()), ksa, len(ks), lik, noise, int(optimise_noise),
                                 C.c_void_p(thd.data_ptr()), C.c_void_p(lld.data_ptr()),
                                 C.c_void_p(infod.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.fgpu_last_error()
    stream.synchronize()
    return float(lld.item()), int(infod.item())


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 63, 65, 300, NOALLOC_MAX_N])
@pytest.mark.parametrize("lik", [0, 1])
@pytest.mark.parametrize("optimise_noise", [False, True])
def test_noalloc_matches_the_context_entry_point_on_two_calls(n, lik, optimise_noise, lib):
    """Sizes from one point up to the scratch limit, where K, the log-det
    parts and the solve vector fill their fixed slots exactly; with the noise
    as the last parameter when it is optimised."""
    torch = pytest.importorskip("torch")
    from fgpu import Engine
    X, y, mu, ks = _problem(n, 5, seed=40 + lik + 7 * n)
    noise = 1e-6
    eng = Engine(X, y, mu, ks, lik, noise, optimise_noise)
    rng = np.random.default_rng(3 + n)
    stream = torch.cuda.Stream()
    for call in range(2):   # the second call reuses the static scratch left by the first
        th = rng.uniform(0.0, 1.0, size=eng.ntheta)
        if optimise_noise:
            # read from theta, not the fixed noise: a value the context's
            # 1e-6 cannot stand in for, kept large enough that K is well
            # conditioned (the two paths round differently)
            th[-1] = rng.uniform(3e-6, 3e-5)
        want, winfo = eng.loglik(th)
        got, ginfo = _call_noalloc(lib, torch, X, y, mu, ks, lik, noise, optimise_noise, th, stream)
        assert ginfo == winfo == 0, (call, ginfo, winfo)
        if n == 1 and lik == 1:
            # one point: the profiled variance is 0 up to rounding, so ll is
            # +inf or a large positive number in either implementation
            assert got > 30 and want > 30
        else:
            assert abs(got - want) <= 1e-9 * abs(want) + 1e-12, (call, got, want)


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    X, y, mu, ks = _problem(NOALLOC_MAX_N + 1, 3, seed=1)
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    ksa = (C.c_int * len(ks))(*ks)
    rc = lib.fgpu_loglik_noalloc(NOALLOC_MAX_N + 1, 3, dummy, dummy, dummy, ksa, len(ks), 0, 1e-6, 0, dummy,
                                 dummy, dummy, None)
    assert rc == -1
    assert b"exceeds the fixed scratch limit" in lib.fgpu_last_error()
