"""The device exponential every kernel-matrix entry goes through (a
fixed-point evaluation on the integer pipes) against the host libm
(numpy.exp): within 1 ulp everywhere the entries live, and IEEE behaviour at
the range ends (1 for tiny arguments, gradual underflow, 0 below -745.13,
NaN propagated)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev_exp(lib, x):
    from fgpu import _lib
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    _lib.check(lib.fgpu_diag_exp(x.ctypes.data_as(_lib.c_double_p), y.ctypes.data_as(_lib.c_double_p), x.size))
    return y


def _ulps(y, ref):
    return np.abs(y - ref) / np.spacing(np.abs(ref))


def test_exp_within_one_ulp_of_libm(lib):
    rng = np.random.default_rng(11)
    x = np.concatenate([
        rng.uniform(-40.0, 0.0, 400000),          # kernel entries exp(-E/2), E >= 0
        rng.uniform(-745.13, 0.0, 200000),        # the whole range, subnormal results included
        rng.uniform(-1e-3, 0.0, 50000),           # near 1
        -np.logspace(-300, 2.87, 20000),          # magnitudes across the exponent range
        rng.uniform(0.0, 1e-12, 1000),            # rounding can make an argument slightly positive
    ])
    y = _dev_exp(lib, x)
    ref = np.exp(x)
    u = _ulps(y, ref)
    # libm is itself within ~0.5 ulp of exact, so 1 ulp between the two allows
    # results rounded to the other neighbour of a near-midpoint value
    assert np.max(u) <= 1.0, (np.max(u), x[np.argmax(u)])
    assert np.mean(u > 0) < 0.02


def test_exp_range_ends(lib):
    x = np.array([0.0, -0.0, -1e-300, -5e-324, -1e-17, -1.0, -708.39, -708.5, -720.0, -744.4,
                  -745.13, -745.14, -746.0, -1e300, -np.inf, np.nan, 1e-14])
    y = _dev_exp(lib, x)
    ref = np.exp(x)
    assert np.all((y == ref) | (_ulps(y, ref) <= 1.0) | (np.isnan(y) & np.isnan(ref))), list(zip(x, y, ref))
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == 1.0 and y[3] == 1.0
    assert y[11] == 0.0 and y[12] == 0.0 and y[13] == 0.0 and y[14] == 0.0 and np.isnan(y[15])
    assert 0.0 < y[10] < 1e-323   # gradual underflow reaches the smallest subnormal


def _dev_exp_fixed(lib, E, e):
    import ctypes as C
    from fgpu import _lib
    E = np.ascontiguousarray(E, dtype=np.uint64)
    y = np.empty(E.size)
    _lib.check(lib.fgpu_diag_exp_fixed(E.ctypes.data_as(C.POINTER(C.c_ulonglong)), e,
                                       y.ctypes.data_as(_lib.c_double_p), E.size))
    return y


@pytest.mark.parametrize("e", [-40, -58, -69])
def test_build_exp_within_one_ulp(lib, e):
    """exp(-E 2^e) for exact integers E (the build's leaf-scale form), against
    the host's extended-precision exp of the exactly represented argument."""
    rng = np.random.default_rng(20 - e)
    top = min(61, 10 - e)                      # arguments up to ~2^10
    bits = rng.integers(0, top, size=300000)
    E = (rng.integers(0, 2 ** 62, size=bits.size, dtype=np.uint64) >> (62 - bits).astype(np.uint64))
    E = np.concatenate([E, np.array([0, 1, 2, 3, 2 ** 20, (2 ** 61) - 1], dtype=np.uint64)])
    E = E[(E.astype(np.float64) * 2.0 ** e) < 740]
    y = _dev_exp_fixed(lib, E, e)
    x = -(E.astype(np.longdouble) * np.longdouble(2.0) ** e)   # exact in a 64-bit or wider significand
    ref = np.exp(x).astype(np.float64)
    ok = ref > 0
    u = np.abs(y[ok] - ref[ok]) / np.spacing(ref[ok])
    assert np.max(u) <= 1.0, (np.max(u), E[ok][np.argmax(u)])
    assert y[E == 0][0] == 1.0
