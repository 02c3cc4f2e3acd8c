"""The FP32 distance bound every FP32 decision of the library rests on
(bound32, fk_internal.cuh): with d32 the FP32 direct form of the f32 copies
of a row and a centre (t = x32 - c32 rounded, acc = fma(t, t, acc)), and e an
upper bound of ||x - x32|| + ||c - c32||, the interval [d32 - b, d32 + b],
b = bound32(d32, e, d), holds both the exact squared distance of the
original values and the FP64 direct form the reference computes.

Checked with exact rational arithmetic: every FP32 operation of the kernels
(round to nearest, fused multiply-add, upward rounding) is emulated exactly,
on rows of several scales and dimensions, with f64 inputs whose f32
roundings are as large as they get."""
import math
from fractions import Fraction

import numpy as np
from exact32 import exponent, f32, round32


def _bound32(d32, ec, d):
    """bound32, operation by operation (fk_internal.cuh)."""
    u = lambda q: round32(q, "u")  # noqa: E731
    dd = d32 if d32 > 0 else Fraction(0)
    if dd > 0:
        h = math.floor(exponent(dd) / 2)
        sq2 = u(u(dd * Fraction(2) ** (-h)) + Fraction(2) ** h)
    else:
        sq2 = Fraction(0)
    e = u(Fraction(d + 4) * Fraction(2) ** -23 * dd)
    e = u(e + u(sq2 * ec))
    e = u(e + u(3 * u(ec * ec)))
    c101 = Fraction(float(np.float32(1.01)))
    return u(u(e * c101) + Fraction(float(np.float32(1e-30))))


def _check(x, c):
    d = len(x)
    x32 = [f32(v) for v in x]
    c32 = [f32(v) for v in c]
    acc = Fraction(0)
    for a, b in zip(x32, c32):
        t = round32(a - b, "n")
        acc = round32(t * t + acc, "n")  # fma: one rounding
    ex = round32(Fraction(math.sqrt(float(sum((Fraction(float(v)) - w) ** 2 for v, w in zip(x, x32))))), "u")
    ec = round32(Fraction(math.sqrt(float(sum((Fraction(float(v)) - w) ** 2 for v, w in zip(c, c32))))), "u")
    # the sqrt above is rounded to nearest in f64: widen by one part in 2^50 to keep it an upper bound
    ex = round32(ex * (1 + Fraction(1, 2 ** 50)), "u")
    ec = round32(ec * (1 + Fraction(1, 2 ** 50)), "u")
    b = _bound32(acc, round32(ex + ec, "u"), d)
    exact = sum((Fraction(float(p)) - Fraction(float(q))) ** 2 for p, q in zip(x, c))
    d64 = 0.0
    for p, q in zip(x, c):
        t = float(p) - float(q)
        d64 = d64 + t * t  # the reference's FP64 direct form (IEEE round to nearest)
    assert acc - b <= exact <= acc + b, (float(acc), float(b), float(exact))
    assert acc - b <= Fraction(d64) <= acc + b


def test_bound32_holds_on_rounded_f64_rows():
    rng = np.random.default_rng(17)
    for d in (1, 3, 16, 64):
        for scale in (1e-3, 1.0, 37.0, 1e4):
            for _ in range(6):
                x = rng.normal(size=d) * scale
                c = x + rng.normal(size=d) * scale * rng.choice([1e-6, 1e-2, 1.0])
                _check(x, c)


def test_bound32_holds_when_the_rows_are_f32_values():
    # the mixed forms' f32 rows: no input rounding on the row, the centre's only
    rng = np.random.default_rng(18)
    for d in (8, 128):
        for _ in range(8):
            x = rng.normal(size=d).astype(np.float32).astype(np.float64) * 20
            c = x + rng.normal(size=d) * 0.3
            _check(x, c)
