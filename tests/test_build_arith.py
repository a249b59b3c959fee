"""CPU restatements of the tensor-core kernel-matrix build's per-entry integer
arithmetic (csrc/build_tc.cu, csrc/iexp.cuh), checked against exact
arithmetic.

* The level assembly from magic-add bits: for level sums |S_L| < 2^22 the
  float S_L + 1.5 2^23 carries S_L in its bits, adjacent levels pair up in 32
  bits and two constants remove the offsets; the result must equal the
  direct integer assembly W = round(sum_L S_L 2^(u - 16 - 8 L)) for every
  scale u the build uses, and the bound 7 x 36 x 2^14 < 2^22 must hold for
  the leaves that take this path.
* The leaf-scale exponential exp(-E 2^e) with two 1024-entry tables and a
  degree-2 polynomial: Python integers mirror the device code step by step
  (64 x 64-bit high products, 32 x 32-bit products, shifts) and the result is
  compared with the correctly rounded value from 50-digit arithmetic.
"""
import random
import struct

import numpy as np
import pytest

M64 = (1 << 64) - 1


def _level_bits(S):
    f = np.asarray(S, dtype=np.float32) + np.float32(12582912.0)
    return f.view(np.uint32).astype(np.uint64)


BIAS_H = (1 << 22) * 0x0101010101 + 0x4B000000 * ((1 << 24) + (1 << 8) + 1)
BIAS_LO = (1 << 22) * 0x010101 + 0x4B000000 * ((1 << 8) + 1)


def _assemble_bits(b, u):
    """assemble_w_bits: b[L] are the magic-add bits of level L (uint32)."""
    b = [int(x) for x in b]
    p01 = (b[0] * 256 + b[1]) & 0xFFFFFFFF
    p23 = (b[2] * 256 + b[3]) & 0xFFFFFFFF
    p56 = (b[5] * 256 + b[6]) & 0xFFFFFFFF
    H = ((p01 << 24) + (p23 << 8) + b[4]) - BIAS_H
    Lo = ((p56 << 8) + b[7]) - BIAS_LO
    return (H << (u - 48)) + ((Lo + (1 << (71 - u))) >> (72 - u))


def _assemble_int(S, u):
    """assemble_w with exact integers."""
    H = sum(int(S[L]) << (32 - 8 * L) for L in range(5))
    Lo = (int(S[5]) << 16) + (int(S[6]) << 8) + int(S[7])
    return (H << (u - 48)) + ((Lo + (1 << (71 - u))) >> (72 - u))


def test_magic_add_range_of_small_leaves():
    # 7 digit pairs per level, at most 36 features, |d_p d_q| <= 2^14
    assert 7 * 36 * (1 << 14) < (1 << 22)
    assert 7 * 37 * (1 << 14) >= (1 << 22)


def test_level_bits_assembly_matches_integer_assembly():
    rng = np.random.default_rng(5)
    lim = 7 * 36 * (1 << 14)
    for trial in range(4000):
        if trial < 8:  # the range ends
            S = np.full(8, lim if trial % 2 else -lim, dtype=np.int64)
            S[trial] = -S[trial]
        else:
            S = rng.integers(-lim, lim + 1, size=8)
        b = _level_bits(S.astype(np.float32))
        for u in range(53, 61):  # u = 60 - ceil(log2 nf), nf <= 128
            assert _assemble_bits(b, u) == _assemble_int(S, u), (S, u)


# ----------------------------------------------------------------------------
# the exponential

mp = pytest.importorskip("mpmath")
mp.mp.dps = 50
L2E64 = int(mp.nint(mp.mpf(2) ** 63 / mp.log(2)))
LN2 = int(mp.nint(mp.log(2) * mp.mpf(2) ** 64))
TAB = [int(mp.nint(mp.mpf(2) ** (mp.mpf(j) / 1024 + 63))) for j in range(1024)]
FINE = [int(mp.nint((mp.mpf(2) ** (mp.mpf(k) / 2 ** 20) - 1) * mp.mpf(2) ** 64)) for k in range(1024)]


def _hi(a, b):
    return (a * b) >> 64


def _bits_to_double(q):
    return struct.unpack("<d", struct.pack("<Q", q))[0]


def _exp_model(E, e):
    """iexp_fixed_tab for 64 <= K0 < 192."""
    if E == 0:
        return 1.0
    K0 = 63 - e
    plo, phi = (E * L2E64) & M64, _hi(E, L2E64)
    if K0 >= 128:
        yi, yf = 0, (phi if K0 == 128 else phi >> (K0 - 128))
    else:
        yi = phi >> (K0 - 64)
        yf = plo if K0 == 64 else (((plo >> (K0 - 64)) | (phi << (128 - K0))) & M64)
    if yi >= 1100:
        return 0.0
    m = yi + (1 if yf else 0)
    f = (-yf) & M64
    j, k, s = f >> 54, (f >> 44) & 1023, f & ((1 << 44) - 1)
    t = _hi(s << 20, LN2) >> 20
    th = t >> 12
    assert th < 1 << 32
    eps = t + ((th * th) >> 41)
    dk = FINE[k]
    assert (dk >> 22) < 1 << 32 and (eps >> 12) < 1 << 32
    de = ((dk >> 22) * (eps >> 12)) >> 30
    p = (1 << 63) + ((dk + eps + de) >> 1)
    assert p < 1 << 64
    Z = _hi(TAB[j], p)
    top = Z >> 63
    sh = 10 + top
    be = 1023 + top - m
    if be >= 1:
        mant = (Z + (1 << (sh - 1))) >> sh
        return _bits_to_double((be << 52) + mant - (1 << 52))
    tot = sh + 1 - be
    if tot > 64:
        return 0.0
    mant = (Z >> 63) if tot == 64 else ((Z + (1 << (tot - 1))) >> tot)
    return _bits_to_double(mant)


def _ulps(a, b):
    ia = struct.unpack("<q", struct.pack("<d", a))[0]
    ib = struct.unpack("<q", struct.pack("<d", b))[0]
    return abs(ia - ib)


@pytest.mark.parametrize("e", [-40, -58, -69, -100])
def test_two_table_exponential_within_one_ulp(e):
    rnd = random.Random(100 - e)
    worst, off = 0, 0
    n = 4000
    for _ in range(n):
        top = rnd.uniform(-60.0, 9.5)  # E 2^e from 2^-60 to ~720
        E = int(2.0 ** (top - e) * rnd.uniform(1.0, 2.0))
        if E <= 0 or E >= 1 << 62:
            continue
        x = mp.mpf(E) * mp.mpf(2) ** e
        if x > 740:
            continue
        u = _ulps(_exp_model(E, e), float(mp.exp(-x)))
        worst = max(worst, u)
        off += u > 0
    assert worst <= 1
    assert off < 0.03 * n
    assert _exp_model(0, e) == 1.0
