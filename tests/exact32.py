"""Exact f32 rounding of rationals, for the CPU tests that restate the
kernels' FP32 arithmetic operation by operation (round to nearest-even or
toward +inf, normal and subnormal ranges)."""
from fractions import Fraction

import numpy as np

F32_MAX = Fraction(2) ** 127 * (2 - Fraction(1, 2 ** 23))
F32_OVERFLOW = Fraction(10) ** 40  # stands for inf: the tests stay far below it


def exponent(a):
    """floor(log2(a)) of a positive rational."""
    e = a.numerator.bit_length() - a.denominator.bit_length()
    return e - 1 if Fraction(2) ** e > a else e


def round32(q, mode="n"):
    """q rounded to an f32 value: 'n' nearest-even, 'u' toward +inf."""
    if q == 0:
        return Fraction(0)
    sign = 1 if q > 0 else -1
    a = abs(q)
    ue = max(exponent(a), -126) - 23
    s = a / Fraction(2) ** ue
    i = s.numerator // s.denominator
    r = s - i
    if mode == "n":
        if r > Fraction(1, 2) or (r == Fraction(1, 2) and i % 2 == 1):
            i += 1
    elif mode == "u":
        if sign > 0 and r > 0:
            i += 1
    else:
        raise ValueError(mode)
    out = sign * i * Fraction(2) ** ue
    return out if abs(out) <= F32_MAX else F32_OVERFLOW * sign


def f32(x):
    """The f32 nearest to x, exactly."""
    return Fraction(float(np.float32(x)))
