"""The exact level sums of the split-integer products, on the CPU.

Every tensor-core contraction of the engine multiplies balanced 8-bit digits
(d in [-128, 127], so |d_p d_q| <= 2^14) and accumulates in fp32 in TMEM;
level l sums the (at most 7) digit-plane pairs p + q = l over the
contraction.  These tests restate, with numpy integers, the bounds and the
conversion the kernels rely on (csrc/tc_common.cuh: `level_bits`,
`level_bits_to_w64`, `levels_to_w64`, `small_f2i`):

* every partial sum stays below 2^24, so the fp32 accumulation is exact, for
  every contraction length of the factorisation (trailing update 128, half
  couplings 64, quarter couplings 32; the kernel-matrix build's bound is in
  test_build_arith.py);
* the magic add x + 1.5 2^23 carries x exactly for |x| < 2^22, and the
  paired-bits assembly equals the direct sum of x_l 256^(6-l);
* the quarter couplings (length 32) are always inside that range, the half
  couplings (64) and the trailing update (128) are not, which is why those
  two check the raw sums (|x| < 2^22 for the whole warp group) and fall back
  to the float-to-int conversion otherwise.
"""
import numpy as np
import pytest

M64 = (1 << 64) - 1
MAGIC = np.float32(12582912.0)  # 1.5 2^23
BIAS = (1 << 22) * 0x0001010101010101 + 0x4B000000 * ((1 << 40) + (1 << 24) + (1 << 8) + 1)


def _worst_level_sum(k):
    """max |level sum| for a contraction of length k: 7 pairs, 2^14 each"""
    return 7 * k * (1 << 14)


@pytest.mark.parametrize("k", [32, 64, 128])
def test_fp32_accumulation_is_exact(k):
    assert _worst_level_sum(k) < (1 << 24)


def test_which_contractions_need_the_range_check():
    assert _worst_level_sum(32) < (1 << 22)  # quarter couplings: always magic
    assert _worst_level_sum(64) >= (1 << 22)  # half couplings: checked
    assert _worst_level_sum(128) >= (1 << 22)  # trailing update: checked


def _bits(x):
    f = np.asarray(x, dtype=np.float32) + MAGIC
    return f.view(np.uint32).astype(np.uint64)


def _w_from_bits(b):
    """level_bits_to_w64 with Python integers (32-bit products wrap)"""
    b = [int(v) for v in b]
    p01 = (b[0] * 256 + b[1]) & 0xFFFFFFFF
    p23 = (b[2] * 256 + b[3]) & 0xFFFFFFFF
    p45 = (b[4] * 256 + b[5]) & 0xFFFFFFFF
    w = (p45 * 256 + b[6]) & M64
    w = (w + (p23 << 24)) & M64
    w = (w + (p01 << 40)) & M64
    w = (w - BIAS) & M64
    return w - (1 << 64) if w >> 63 else w


def _w_direct(S):
    return sum(int(S[l]) << (8 * (6 - l)) for l in range(7))


def _w_f2i(S):
    """levels_to_w64: the wrapping sum (the fallback after float-to-int)"""
    w = 0
    for l in range(7):
        w = (w + ((int(S[l]) & M64) << (8 * (6 - l)))) & M64
    return w - (1 << 64) if w >> 63 else w


def test_magic_add_is_exact_below_2_22():
    x = np.arange(-(1 << 22), 1 << 22, 997, dtype=np.int64)
    x = np.concatenate([x, [-(1 << 22), (1 << 22) - 1, -1, 0, 1]])
    b = _bits(x.astype(np.float32))
    assert np.all((b >> 23) == (0x4B000000 >> 23))
    assert np.array_equal(b.astype(np.int64) - 0x4B000000 - (1 << 22), x)


def test_paired_bits_assembly_matches_the_direct_sum():
    rng = np.random.default_rng(11)
    lim = (1 << 22) - 1
    for trial in range(3000):
        if trial < 14:  # the range ends, one level at a time
            S = np.full(7, lim if trial % 2 else -lim, dtype=np.int64)
            S[trial % 7] = -S[trial % 7]
        else:
            S = rng.integers(-lim, lim + 1, size=7)
        W = _w_direct(S)
        if abs(W) >= 1 << 62:
            continue
        assert _w_from_bits(_bits(S.astype(np.float32))) == W, S
        assert _w_f2i(S) == W, S


@pytest.mark.parametrize("k", [32, 64, 128])
def test_contraction_level_sums_and_the_range_check(k):
    """Random and extreme digit planes, level sums formed exactly; the raw
    range check (|x| < 2^22 over a group) picks the magic path only where
    the magic path is exact, and either path gives the same W."""
    rng = np.random.default_rng(k)
    used_magic = used_f2i = 0
    for trial in range(200):
        if trial == 0:
            A = np.full((7, k), -128, dtype=np.int64)  # the worst level sums
            B = np.full((7, k), -128, dtype=np.int64)
        else:
            A = rng.integers(-128, 128, size=(7, k))
            B = rng.integers(-128, 128, size=(7, k))
        S = np.zeros(7, dtype=np.int64)
        for p in range(7):
            for q in range(7 - p):
                S[p + q] += int(A[p] @ B[q])
        raw = S.astype(np.float32)
        assert np.array_equal(raw.astype(np.int64), S)  # fp32 exact
        # random top digits give |W| beyond 2^63, which no factor entry
        # reaches; both assemblies are exact modulo 2^64 regardless
        W = _w_direct(S) & M64
        if float(np.max(np.abs(raw))) < 4194304.0:
            used_magic += 1
            assert _w_from_bits(_bits(raw)) & M64 == W
        else:
            used_f2i += 1
        assert _w_f2i(raw.astype(np.int64)) & M64 == W
    assert used_magic > 0
    if k == 32:
        assert used_f2i == 0
    else:
        assert used_f2i > 0  # the all -128 planes leave the magic range
