"""CPU emulation of the compensated FP32 arithmetic the kernels use in place
of FP64 (FP64 runs at 1/64 of the FP32 rate on GB300): the scaled two-part
squares of micro_window_kernel (csrc/nz_canonical.cu: scaled_split,
add_square) and the TwoSum accumulators of the convolutions (ConvAcc<1>,
csrc/nz_conv_tc.cu: two_sum_add).  numpy float32 operations are IEEE
round-to-nearest like the device's __fadd_rn / __fmul_rn; fmaf is emulated
exactly with rationals.  The GPU tests check the kernels themselves against
the oracle at the scales they reach (tests/test_gpu_ensemble.py); these pin
the method at the scale exponents and magnitudes they do not."""
import random
from fractions import Fraction

import numpy as np
import pytest

f32 = np.float32


def fmaf(a, b, c):
    """a * b + c rounded once to float32 (exact rational, then nearest)."""
    exact = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    r = f32(float(exact))  # may double-round; pick the nearest neighbour
    cands = (r, np.nextafter(r, f32(np.inf)), np.nextafter(r, f32(-np.inf)))
    return min(cands, key=lambda v: abs(Fraction(float(v)) - exact))


def scaled_split(x, e):
    """|d| (< 2^96) times 2^-e as (yh, yl): its top 24 significant bits and
    the next 24, both exact in FP32 (scaled_split in nz_canonical.cu)."""
    nb = x.bit_length()
    s2 = nb - 48 if nb > 48 else 0
    y = x >> s2
    sh = nb - s2 - 24 if nb > 24 else 0
    top = y >> sh
    k = s2 - e
    yh, yl = f32(top * 2.0 ** (sh + k)), f32((y - (top << sh)) * 2.0 ** k)
    assert float(yh) == top * 2.0 ** (sh + k) and float(yl) == (y - (top << sh)) * 2.0 ** k
    return yh, yl


def add_square(s, c, yh, yl):
    """(s, c) += (yh + yl)^2 as add_square in nz_canonical.cu."""
    p = f32(yh * yh)
    pe = fmaf(yh, yh, -p)
    cross = fmaf(f32(2) * yh, yl, f32(yl * yl))
    t = f32(s + p)
    bp = f32(t - s)
    err = f32(f32(s - f32(t - bp)) + f32(p - bp))
    return t, f32(c + f32(err + f32(pe + cross)))


def two_sum_add(s, c, x):
    t = f32(s + x)
    bp = f32(t - s)
    return t, f32(c + f32(f32(s - f32(t - bp)) + f32(x - bp)))


def scale_exponent(N, power):
    """e3 / e4 of micro_window_kernel: |d| 2^-e <= 2^40 for d < N^power."""
    nbits = int(N).bit_length()
    return max(0, min(power * nbits, 96) - 40)


@pytest.mark.parametrize('N,power', [(100, 3), (16384, 3), (16384, 4), (65536, 4), (115600, 4),
                                     (2 ** 21 - 1, 3), (2 ** 21 - 1, 4)])
def test_scaled_fp32_squares(N, power):
    """Sum of d^2 over a thread's runs to ~1e-13 relative, for deviations up
    to the statistic's bound (m3 < N^3, m4 < N^4 and < 2^96) down to 1, with
    the squares and sums inside FP32's normal range."""
    rng = random.Random(N * 10 + power)
    e = scale_exponent(N, power)
    bound = min(N ** power, 2 ** 96)
    for spread in (bound, bound // 1000 + 1, 1000, 1):
        s = c = f32(0)
        exact = 0
        for _ in range(400):
            d = rng.randrange(spread + 1)
            yh, yl = scaled_split(d, e)
            if d:
                assert abs(float(yh)) >= 2.0 ** -126 or float(yh) == 0.0
            s, c = add_square(s, c, yh, yl)
            exact += d * d
        assert np.isfinite(s) and np.isfinite(c)
        got = (Fraction(float(s)) + Fraction(float(c))) * Fraction(2) ** (2 * e)
        if exact == 0:
            assert got == 0
        else:
            assert abs(got - exact) / exact < 1e-12, (N, power, spread)


def test_two_sum_accumulator_matches_exact_sum():
    """The FP32 (sum, compensation) pair of the convolutions adds hundreds
    of FP32 chunk sums of very different sizes as accurately as FP64 does."""
    rng = np.random.default_rng(3)
    xs = (rng.random(500) * 10.0 ** rng.integers(-8, 8, 500)).astype(np.float32)
    s = c = f32(0)
    for x in xs:
        s, c = two_sum_add(s, c, x)
    exact = sum(Fraction(float(x)) for x in xs)
    got = Fraction(float(s)) + Fraction(float(c))
    assert abs(got - exact) / exact < 1e-13
    # a plain FP32 running sum of the same values is ~1e-8 off
    plain = f32(0)
    for x in xs:
        plain = f32(plain + x)
    assert abs(Fraction(float(plain)) - exact) / exact > 1e-10


def split_value(q):
    """An integer q < 2^48 as (qh, ql): q rounded toward zero to 24
    significant bits and the exact remainder (split_u64 / split_u32 in
    nz_canonical.cu)."""
    nb = q.bit_length()
    sh = nb - 24 if nb > 24 else 0
    qh = (q >> sh) << sh
    return f32(qh), f32(q - qh)


def dot2_add(s, c, wh, wl, qh, ql):
    """One compensated term of conv_m2_comp_kernel (Dot2Acc.add):
    TwoProduct, and Fast2Sum on the operands ordered by size (all >= 0)."""
    ph = f32(wh * qh)
    eh = fmaf(wh, qh, -ph)
    a, b = max(s, ph), min(s, ph)
    t = f32(a + b)
    e = f32(b - f32(t - a))
    c = f32(c + f32(e + eh))
    c = fmaf(wh, ql, c)
    c = fmaf(wl, qh, c)
    return t, c


@pytest.mark.parametrize('L,rows', [(256, 2800), (1024, 3000)])
def test_compensated_m2_products_reach_5e_11(L, rows):
    """The m2 convolution of one run over a binomial-shaped band as
    conv_m2_comp_kernel does it -- FP64 weights split into FP32 hi + lo, m2
    values (up to N^2 / 4) split into exact FP32 parts, compensated products
    and sums over every chunk of 128 rows that meets the core (weights >=
    e^-8 of the largest), plain FP32 products over chunks entirely in the
    tails, added into the running sum chunk by chunk -- comes within 5e-11
    relative of the exact dot product of the FP64 weights: what the
    susceptibility curve needs to stay within 1e-6 absolute of FP64 at
    L = 1024 (m2 / N up to ~2e4).  Plain FP32 products summed in FP32 are
    ~1e-7 off."""
    rng = np.random.default_rng(L)
    N = L * L
    n = np.arange(rows)
    sigma = rows / 15.5  # the FP32 band: +-7.75 standard deviations
    w = np.exp(-0.5 * ((n - rows / 2) / sigma) ** 2)
    w /= w.sum()
    core = w >= w.max() * np.exp(-8.0)
    hi = rng.integers(1, N * N // 4, rows // 4 + 1)
    q = [int(x) for x in np.repeat(hi, 4)[:rows] + rng.integers(0, 1000, rows)]
    exact = sum(Fraction(float(wi)) * qi for wi, qi in zip(w, q))
    s = c = f32(0)
    plain = f32(0)
    for c0 in range(0, rows, 128):  # chunks of 128 rows
        compensated = bool(core[c0:c0 + 128].any())
        tail = f32(0)
        for i in range(c0, min(rows, c0 + 128)):
            wi, qi = w[i], q[i]
            wh = f32(wi)
            wl = f32(float(wi) - float(wh))
            qh, ql = split_value(qi)
            assert int(qh) + int(ql) == qi
            if compensated:
                s, c = dot2_add(s, c, wh, wl, qh, ql)
            else:
                tail = fmaf(wh, f32(qh + ql), tail)
            plain = fmaf(wh, f32(qi), plain)
        if not compensated:  # flush_tail: Fast2Sum into the running sum
            a, b = max(s, tail), min(s, tail)
            t = f32(a + b)
            c, s = f32(c + f32(b - f32(t - a))), t
    got = Fraction(float(s)) + Fraction(float(c))
    assert abs(got - exact) / exact < 5e-11
    assert abs(Fraction(float(plain)) - exact) / exact > 1e-9
