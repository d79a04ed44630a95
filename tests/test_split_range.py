"""The split Gram's magnitude range, restated on the CPU.

oz_gram.cu scales each 64-row chunk's exact level sums by powers of two and
adds them into FP32 (hi, lo) pairs, so its accuracy holds only while the
scaled products stay inside FP32's range; include/lobpcg_gb300.h states the
range (products of two columns' chunk maxima between 2^-120 and 2^100).
This test restates the kernel's arithmetic for FP64 inputs -- the chunk
exponent, the 32-bit fixed point and its four 8-bit digits (oz_digits4x8_u),
the exact level sums, the scales 2^(E - 1030) (zero outside [904, 1157]),
the two-sum of level 0 into hi, the Horner sum of levels 1-3 into lo, the
renormalisation every 8 chunks -- with numpy FP32 operations, and checks it
against the exact sum (fractions) and the stated error bound inside the
range, and that it fails outside (which is why the range is documented).
"""
from fractions import Fraction

import numpy as np

f32 = np.float32
MAG = f32(1.5 * 2.0 ** 23)


def _bexp(v):
    return int((np.float64(v).view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF))


def _fixed(v, E, F=32):
    b = np.float64(v).view(np.uint64)
    be = int((b >> np.uint64(52)) & np.uint64(0x7FF))
    if be == 0:
        return 0
    M = int(b & np.uint64(0xFFFFFFFFFFFFF)) | (1 << 52)
    sh = 53 - F + (E - be)
    return 0 if sh >= 64 else (M + (1 << (sh - 1))) >> sh


def _digits(v, E):
    U = _fixed(v, E)
    s = -1.0 if v < 0 else 1.0
    h, l = f32(s * (U >> 16)), f32(s * (U & 0xFFFF))
    d0 = f32(f32(h * f32(2.0 ** -8) + MAG) - MAG)
    d1 = f32(h - f32(256.0) * d0)
    d2 = f32(f32(l * f32(2.0 ** -8) + MAG) - MAG)
    d3 = f32(f32(f32(l - f32(256.0) * d2) + MAG) - MAG)
    return [float(d0), float(d1), float(d2), float(d3)]


def _scale(E):
    return f32(2.0 ** (E - 1030)) if 904 <= E <= 1157 else f32(0.0)


def _fma32(a, b, c):
    # a b is exact in FP64; the sum rounds once to FP64 and then to FP32 (a
    # double rounding the kernel's fmaf does not have: far below the bound)
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def split_gram_entry(x, y):
    hi, lo = f32(0), f32(0)
    with np.errstate(over="ignore", invalid="ignore"):
        for c, r0 in enumerate(range(0, len(x), 64)):
            xs, ys = x[r0:r0 + 64], y[r0:r0 + 64]
            Ex, Ey = max(map(_bexp, xs)), max(map(_bexp, ys))
            dx, dy = [_digits(v, Ex) for v in xs], [_digits(v, Ey) for v in ys]
            S = [f32(sum(dx[r][t] * dy[r][L - t] for r in range(len(xs)) for t in range(L + 1)))
                 for L in range(4)]
            rest = S[3]
            for L in (2, 1):
                rest = _fma32(rest, f32(2.0 ** -8), S[L])
            fij = f32(_scale(Ex) * _scale(Ey))
            a = f32(S[0] * fij)
            s = f32(hi + a)
            bv = f32(s - hi)
            err = f32(f32(hi - f32(s - bv)) + f32(a - bv))
            hi = s
            lo = _fma32(rest, f32(fij * f32(2.0 ** -8)), f32(lo + err))
            if c % 8 == 7:
                s = f32(hi + lo)
                bv = f32(s - hi)
                lo = f32(f32(hi - f32(s - bv)) + f32(lo - bv))
                hi = s
    return float(hi) + float(lo)


def _bound(x, y):
    b = 0.0
    for r0 in range(0, len(x), 64):
        xs, ys = x[r0:r0 + 64], y[r0:r0 + 64]
        b += 2.0 ** -29 * 64 * np.abs(xs).max() * np.abs(ys).max() + 2.0 ** -30 * abs(xs @ ys)
    return b + 2.0 ** -50 * float(np.abs(x) @ np.abs(y))


def _exact(x, y):
    return float(sum(Fraction(a) * Fraction(b) for a, b in zip(x, y)))


def test_accurate_inside_the_stated_range():
    rng = np.random.default_rng(0)
    n = 64 * 24 + 17
    x0, y0 = rng.standard_normal(n), rng.standard_normal(n)
    for sx, sy in ((0, 0), (-58, -58), (48, 48), (-60, 50), (30, -40)):
        x, y = x0 * 2.0 ** sx, y0 * 2.0 ** sy
        g = split_gram_entry(x, y)
        assert np.isfinite(g)
        assert abs(g - _exact(x, y)) <= _bound(x, y), (sx, sy)


def test_inaccurate_outside_it():
    rng = np.random.default_rng(1)
    n = 64 * 8
    x0, y0 = rng.standard_normal(n), rng.standard_normal(n)
    small = split_gram_entry(x0 * 2.0 ** -70, y0 * 2.0 ** -70)    # products near 2^-136
    assert abs(small - _exact(x0 * 2.0 ** -70, y0 * 2.0 ** -70)) > _bound(x0 * 2.0 ** -70,
                                                                          y0 * 2.0 ** -70)
    large = split_gram_entry(x0 * 2.0 ** 70, y0 * 2.0 ** 70)      # products near 2^144
    assert not np.isfinite(large)


# ------------------------------------------------ the update (oz_xc.cu)
def split_update_entry(xrow, ccol):
    """Y_ij of oz_xc restated: the row's and the column's scales, six 7-bit
    digits of each value (three exact 14-bit parts of the 42-bit fixed point
    for X, balanced digits for C), the levels t + u <= 5 summed exactly, the
    integer rounded once to FP64 and scaled by 2^(er + ec - 2093)."""
    from tests.test_split_digits import bexp64, fixed64, update_c_digits, update_x_digits
    er, ec = max(map(bexp64, xrow)), max(map(bexp64, ccol))
    if er == 0 or ec == 0:
        return 0.0
    T = 0
    for xv, cv in zip(xrow, ccol):
        _, dx = update_x_digits(xv, er)
        dc = update_c_digits(fixed64(cv, ec, F=42), cv < 0)
        for t in range(6):
            for u in range(6 - t):
                T += int(dx[t]) * int(dc[u]) * 128 ** (5 - t - u)
    return float(T) * 2.0 ** (er + ec - 2093)


def test_update_restated_meets_its_bound_over_the_fp64_range():
    """|Y - X C| <= h 2^-38 rowmax|X| colmax|C| (plus the final rounding):
    the update recombines in integers and scales on the FP64 exponent field,
    so the bound holds across the FP64 range, unlike the Gram's FP32 pairs."""
    rng = np.random.default_rng(5)
    h = 64
    for sx, sc in ((0, 0), (-300, 250), (400, -380), (-60, -60), (90, 90)):
        for _ in range(3):
            x = rng.standard_normal(h) * np.exp(3 * rng.standard_normal(h)) * 2.0 ** sx
            c = rng.standard_normal(h) * np.exp(3 * rng.standard_normal(h)) * 2.0 ** sc
            y = split_update_entry(x, c)
            ex = _exact(x, c)
            bound = h * 2.0 ** -38 * np.abs(x).max() * np.abs(c).max()
            assert abs(y - ex) <= bound + abs(ex) * 2.0 ** -52, (sx, sc, y, ex)
