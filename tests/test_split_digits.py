"""The digit schemes of the split-operand products, restated on the CPU.

The Gram (oz_gram.cu) cuts every value of a 64-row chunk column into four
8-bit digits relative to the chunk's largest exponent E (oz_digits4x8_* in
oz_common.cuh); the products of digit pairs are summed per level on the
tensor cores in FP32, which is exact only while every level sum stays below
2^24.  These tests restate the digit extraction (FP32 round-to-nearest
steps, emulated exactly in FP64: every intermediate below fits 53 bits) and
the FP64 integer path, and check on adversarial values -- the group maximum,
values just below a power of two, both signs, values many binades below E
-- that
  * every digit is an integer with |d0| <= 256 and |d1|, |d2|, |d3| <= 128
    (FP32 path) or d2 <= 256 (integer path), so it is exact in bf16 (an
    integer of at most 8 significant bits: the FP32 pattern's low 16 bits
    are zero);
  * the digits rebuild the 32-bit fixed point value to within 1/2 unit;
  * the level sums over 64 rows of the worst digits stay below 2^24.
The same for the block update (oz_xc.cu): six 7-bit digits per value of X
(three exact 14-bit parts) and of C (balanced by a bias), rebuilding the
42-bit fixed point exactly, and level sums over 64 terms below 2^22.
"""
import numpy as np
import pytest

MAGIC = 1.5 * 2.0 ** 23


def f32(x):
    return np.float32(x)


def rint32(x):
    """(x + 1.5 2^23) - 1.5 2^23 in FP32, for |x| < 2^22 (x exact in FP64)."""
    return np.float64(f32(np.float64(x) + MAGIC)) - MAGIC


def digits_hl(h, l):
    d0 = rint32(h * 2.0 ** -8)
    d1 = np.float64(f32(h - 256.0 * d0))
    d2 = rint32(l * 2.0 ** -8)
    d3 = rint32(l - 256.0 * d2)
    return [d0, d1, d2, d3]


def digits_f32(v, E):
    scale = 2.0 ** (32 + 1022 - E)
    u = np.float64(f32(np.float64(v) * scale))  # exact: v has 24 bits
    h = rint32(u * 2.0 ** -16)
    l = np.float64(f32(u - 65536.0 * h))
    return u, digits_hl(h, l)


def fixed64(v, E, F=32):
    """round(|v| 2^(F - (E - 1022))) from the bits, as oz_fixed64<F>."""
    b = np.float64(v).view(np.uint64)
    be = int((b >> np.uint64(52)) & np.uint64(0x7FF))
    if be == 0:
        return 0
    M = int(b & np.uint64(0xFFFFFFFFFFFFF)) | (1 << 52)
    sh = 53 - F + (E - be)
    if sh >= 64:
        return 0
    return (M + (1 << (sh - 1))) >> sh


def digits_u(U, neg):
    s = -1.0 if neg else 1.0
    h = s * float(U >> 16)
    l = s * float(U & 0xFFFF)
    return digits_hl(h, l)


def bexp32(v):
    e = int((np.float32(v).view(np.uint32) >> np.uint32(23)) & np.uint32(0xFF))
    return e + 896 if e else 0


def bexp64(v):
    return int((np.float64(v).view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF))


def _is_bf16_exact(d):
    bits = int(np.float32(d).view(np.uint32))
    return (bits & 0xFFFF) == 0


def _adversarial(rng, n):
    base = rng.standard_normal(n)
    vals = list(base)
    for e in (0, 1, -1, 7, -20):
        vals += [np.nextafter(2.0 ** e, 0.0), 2.0 ** e, -(2.0 ** e), 1.5 * 2.0 ** e]
    vals += list(base * 10.0 ** rng.uniform(-12, 0, n))
    return np.array(vals)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_fp32_digits_exact_and_bounded(seed):
    rng = np.random.default_rng(seed)
    v32 = _adversarial(rng, 200).astype(np.float32)
    E = max(bexp32(x) for x in v32)
    for v in v32:
        u, d = digits_f32(v, E)
        assert all(float(x).is_integer() for x in d), (v, d)
        assert abs(d[0]) <= 256 and all(abs(x) <= 128 for x in d[1:]), (v, d)
        assert all(_is_bf16_exact(x) for x in d)
        rebuilt = d[0] * 2.0 ** 24 + d[1] * 2.0 ** 16 + d[2] * 2.0 ** 8 + d[3]
        assert abs(rebuilt - u) <= 0.5, (v, u, rebuilt)


@pytest.mark.parametrize("seed", [3, 4])
def test_fp64_integer_digits_exact_and_bounded(seed):
    rng = np.random.default_rng(seed)
    v64 = _adversarial(rng, 200)
    E = max(bexp64(x) for x in v64)
    for v in v64:
        U = fixed64(v, E)
        assert U <= 2 ** 32
        d = digits_u(U, v < 0)
        assert all(float(x).is_integer() for x in d)
        assert abs(d[0]) <= 256 and abs(d[1]) <= 128 and abs(d[2]) <= 256 and abs(d[3]) <= 128
        assert all(_is_bf16_exact(x) for x in d)
        rebuilt = d[0] * 2.0 ** 24 + d[1] * 2.0 ** 16 + d[2] * 2.0 ** 8 + d[3]
        assert rebuilt == (-U if v < 0 else U)
        # the fixed point is |v| to within half a unit of 2^(E - 1022 - 32)
        assert abs(abs(v) * 2.0 ** (32 - (E - 1022)) - U) <= 0.5


def test_level_sums_below_2_24_over_a_chunk():
    """The worst digits (|d0| = 256, |d1| = |d3| = 128, |d2| = 256 on the
    integer path) on all 64 rows of a chunk: every level L = t + u < 4 sums
    at most 64 * sum_{t+u=L} |d_t| |d_u| < 2^24, so FP32 holds it exactly."""
    dmax = [256, 128, 256, 128]
    for L in range(4):
        worst = 64 * sum(dmax[t] * dmax[L - t] for t in range(L + 1))
        assert worst < 2 ** 24, (L, worst)


# ------------------------------------------------ the update's six 7-bit digits
def update_x_digits(v, E):
    """ozx_digits (oz_xc.cu): the 42-bit fixed point in three 14-bit parts,
    each cut into a rounded 7-bit digit and its remainder."""
    U = fixed64(v, E, F=42)
    s = -1.0 if v < 0 else 1.0
    parts = [U >> 28, (U >> 14) & 0x3FFF, U & 0x3FFF]
    d = []
    for p in parts:
        c = s * float(p)
        a = rint32(c * 2.0 ** -7)
        d += [a, np.float64(f32(c - 128.0 * a))]
    return U, d


def update_c_digits(U, neg, S=6):
    """oz_digits<S> (oz_common.cuh): balanced 7-bit digits by a bias of 64
    on every digit below the top one."""
    bias = sum(64 << (7 * (S - 1 - t)) for t in range(1, S))
    V = U + bias
    d = [V >> (7 * (S - 1))] + [((V >> (7 * (S - 1 - t))) & 127) - 64 for t in range(1, S)]
    return [-x if neg else x for x in d]


@pytest.mark.parametrize("seed", [5, 6])
def test_update_digits_exact_and_bounded(seed):
    rng = np.random.default_rng(seed)
    vals = _adversarial(rng, 150)
    E = max(bexp64(x) for x in vals)
    for v in vals:
        U, d = update_x_digits(v, E)
        assert all(float(x).is_integer() for x in d)
        assert all(abs(x) <= 128 for x in d[0::2]) and all(abs(x) <= 64 for x in d[1::2])
        assert all(_is_bf16_exact(x) for x in d)
        rebuilt = sum(d[t] * 2.0 ** (7 * (5 - t)) for t in range(6))
        assert rebuilt == (-U if v < 0 else U)
        dc = update_c_digits(U, v < 0)
        assert abs(dc[0]) <= 129 and all(abs(x) <= 64 for x in dc[1:])
        assert sum(dc[t] * 2 ** (7 * (5 - t)) for t in range(6)) == (-U if v < 0 else U)


def test_update_level_sums_below_2_22_over_64_columns():
    """h <= 64 contraction terms per output: every kept level L = t + u < 6
    of the update's digit products (X: |d| <= 128 / 64 alternating; C: top
    digit <= 129, the rest <= 64) sums below 2^22, so two levels combine in a
    32-bit integer (S_L 128 + S_{L+1}) as the epilogue does."""
    dx = [128, 64, 128, 64, 128, 64]
    dc = [129, 64, 64, 64, 64, 64]
    for L in range(6):
        worst = 64 * sum(dx[t] * dc[L - t] for t in range(L + 1))
        assert worst < 2 ** 22, (L, worst)
