"""CPU checks of the integer identities the tensor-core kernels rely on.

The kernels cannot be run here, but the arithmetic they depend on for
exactness can: each test restates one identity with numpy int64 and checks
it over random inputs covering the full ranges the kernels admit.

* Balanced base-256 digits of a 55-bit fixed-point value (the 7 fp16 digit
  planes): the reference extraction (peel the low byte as a signed char, 6
  times) against the biased-byte form the panel solve uses (add 128 to each
  of the 6 low byte positions; bytes are digit + 128, the top 16 bits the
  top digit).
* The fp16 construction of a digit: the half with bits 0x6400 + u is
  1024 + u, and subtracting 1152 gives u - 128 exactly.
* The trailing update's drain: W = sum_l S_l 2^(8 (6 - l)) assembled level by
  level as hi 2^24 + lo with levels 4..6 split at 2^24, against the direct
  int64 formula.
"""
import numpy as np


def _reference_digits(F):
    """7 balanced digits, d[0] the top one (the kernels' plane order)."""
    d = np.zeros((7,) + F.shape, dtype=np.int64)
    f = F.copy()
    for p in range(6, 0, -1):
        b = ((f & 0xFF) ^ 0x80) - 0x80  # signed char of the low byte
        d[p] = b
        f = (f - b) >> 8
    d[0] = f
    return d


def _biased_digits(F):
    G = F + 0x808080808080
    d = np.zeros((7,) + F.shape, dtype=np.int64)
    d[0] = G >> 48
    for p in range(1, 7):
        q = 6 - p
        d[p] = ((G >> (8 * q)) & 0xFF) - 128
    return d


def test_biased_byte_digits_match_reference():
    rng = np.random.default_rng(0)
    F = rng.integers(-(1 << 55), (1 << 55) + 1, size=200_000, dtype=np.int64)
    F[:1000] = rng.integers(-300, 301, size=1000)  # small magnitudes and zero
    F[1000] = 1 << 55
    F[1001] = -(1 << 55)
    ref = _reference_digits(F)
    assert np.array_equal(_biased_digits(F), ref)
    # the digits rebuild F and stay in the exactness bounds of the MMA levels
    w = np.array([256 ** (6 - p) for p in range(7)], dtype=np.int64)
    assert np.array_equal((ref * w[:, None]).sum(axis=0), F)
    assert np.all(np.abs(ref[1:]) <= 128) and np.all(np.abs(ref[0]) <= 128)


def test_fp16_digit_from_biased_byte_is_exact():
    u = np.arange(0, 257, dtype=np.uint16)
    h = (u + 0x6400).astype(np.uint16).view(np.float16)
    off = np.array([0x6480], dtype=np.uint16).view(np.float16)[0]
    assert float(off) == 1152.0
    assert np.array_equal((h - off).astype(np.int64), u.astype(np.int64) - 128)


def test_progressive_level_assembly_matches_direct_formula():
    rng = np.random.default_rng(1)
    n = 100_000
    # level l sums at most (l + 1) x 128 products of |d| <= 128 (K = 128)
    S = np.stack([rng.integers(-(l + 1) * (1 << 21), (l + 1) * (1 << 21) + 1, size=n, dtype=np.int64)
                  for l in range(7)])
    # direct: low = S4 2^16 + S5 2^8 + S6, hi = S0 2^24 + ... + S3 + (low >> 24)
    low = S[4] * 65536 + S[5] * 256 + S[6]
    hi_ref = S[0] * 16777216 + S[1] * 65536 + S[2] * 256 + S[3] + (low >> 24)
    lo_ref = low & 0xFFFFFF
    # progressive, as the drain gathers it
    hi = np.zeros(n, dtype=np.int64)
    lo = np.zeros(n, dtype=np.int64)
    for l in range(7):
        if l <= 3:
            hi += S[l] << (8 * (3 - l))
        else:
            k = 8 * (l - 3)
            hi += S[l] >> k
            lo += (S[l] & ((1 << k) - 1)) << (8 * (6 - l))
    assert np.all(lo < 3 * (1 << 24)) and np.all(lo >= 0)
    hi += lo >> 24
    lo &= 0xFFFFFF
    assert np.array_equal(hi, hi_ref) and np.array_equal(lo, lo_ref)


def test_magic_add_conversion_range():
    """x + 1.5 2^23 in float32 keeps an integer x exactly for |x| <= 2^22:
    the bound behind converting the top levels (and every level of a K <= 32
    coupling) without a float-to-int instruction."""
    x = np.concatenate([np.arange(-(1 << 22), -(1 << 22) + 2000), np.arange(-1000, 1001),
                        np.arange((1 << 22) - 2000, (1 << 22) + 1)]).astype(np.float32)
    y = (x + np.float32(12582912.0)).view(np.int32) - 0x4B400000
    assert np.array_equal(y, x.astype(np.int64))
