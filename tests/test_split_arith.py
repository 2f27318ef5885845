"""The number format of the split-precision op-list kernel, restated with exact integers (host
only, no GPU).

Each operand is rounded to 56 bits of its row (left factor) or column (right factor) scale and cut
into 8 signed digits of 7 bits (x = 2^e sum_t d_t 2^(-7(t+1)), |d_t| <= 128, exactly representable
in FP16); a product keeps the digit pairs with t + u <= L and sums them per level t + u.  These
tests pin the two facts the kernel's accuracy rests on:

* every level sum of a 32-term product stays below 2^22, so FP32 accumulators biased by 1.5 2^23
  hold it exactly and one integer subtraction reads it back;
* keeping the pairs up to level 8 (43 products, the kernel's choice) leaves a 32-term product
  within about 2^-56 of (row scale x column scale), the rounding of the operands to 56 bits,
  against about 2^-51 for levels up to 7 (36 products, truncation dominating); with entries
  much smaller than their row's largest, only the former keeps FP64 accuracy relative to them.
"""
import math
from fractions import Fraction

import numpy as np


def digits(x, e):
    """Signed 7-bit digits of x at scale 2^e (|x| < 2^e): round |x| 2^(56-e) to an integer F
    (56 bits), digit 0 = F >> 49 (may reach 128), digit t = (F >> (49 - 7t)) & 127."""
    F = round(abs(Fraction(x)) * 2 ** (56 - e))
    d = [F >> 49] + [(F >> (49 - 7 * t)) & 0x7F for t in range(1, 8)]
    s = -1 if x < 0 else 1
    return [s * v for v in d]


def value(d, e):
    return sum(Fraction(v) * Fraction(2) ** (e - 7 * (t + 1)) for t, v in enumerate(d))


def split_dot(a, b, ea, eb, max_level):
    """sum_i a_i b_i from digit pairs with t + u <= max_level; returns (value, level sums)."""
    da = [digits(x, ea) for x in a]
    db = [digits(x, eb) for x in b]
    levels = [0] * (max_level + 1)
    for xa, xb in zip(da, db):
        for t in range(8):
            for u in range(8):
                if t + u <= max_level:
                    levels[t + u] += xa[t] * xb[u]
    val = sum(Fraction(lv) * Fraction(2) ** (ea + eb - 7 * (l + 2)) for l, lv in enumerate(levels))
    return val, levels


def scale(v):
    m = max(abs(x) for x in v)
    return math.frexp(m)[1] if m else 0  # |x| < 2^e


def test_digits_reconstruct_to_56_bits():
    rng = np.random.default_rng(1)
    for _ in range(200):
        x = float(rng.standard_normal() * 10.0 ** rng.uniform(-5, 5))
        e = math.frexp(abs(x))[1] + int(rng.integers(0, 3))
        d = digits(x, e)
        assert all(abs(v) <= 128 for v in d) and all(abs(v) <= 127 for v in d[1:])
        err = abs(value(d, e) - Fraction(x))
        assert err <= Fraction(2) ** (e - 57)  # half a unit of the 56-bit rounding


def test_level_sums_fit_the_fp32_accumulators():
    rng = np.random.default_rng(2)
    worst = 0
    for _ in range(20):
        a = rng.standard_normal(32)
        b = rng.standard_normal(32)
        a[:] = np.abs(a) * 0.999  # same signs everywhere: the largest level sums
        b[:] = np.abs(b) * 0.999
        _, levels = split_dot(a, b, scale(a), scale(b), 8)
        worst = max(worst, max(abs(v) for v in levels))
    assert worst < 2 ** 22


def test_level_eight_keeps_small_entries_accurate():
    rng = np.random.default_rng(3)
    err7 = err8 = 0.0
    for _ in range(30):
        n = 32
        a = rng.standard_normal(n)
        a[0] = 64.0  # one large entry sets the row scale (a triangular factor's diagonal)
        b = rng.standard_normal(n)
        ea, eb = scale(a), scale(b)
        exact = sum(Fraction(x) * Fraction(y) for x, y in zip(a, b))
        rel = Fraction(2) ** (ea + eb)
        v7, _ = split_dot(a, b, ea, eb, 7)
        v8, _ = split_dot(a, b, ea, eb, 8)
        err7 = max(err7, float(abs(v7 - exact) / rel))
        err8 = max(err8, float(abs(v8 - exact) / rel))
    assert err8 < 2.0 ** -55
    assert err7 > 8 * err8  # the extra level removes the truncation error (about 2^-51)
