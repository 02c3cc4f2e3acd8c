"""The f32 rounding error of an f64 value as the plain f64 assignment's FP32
bounds form it from the value's bits (fk_prefilter.cu round_err): for v in
the f32 normal range, |v - fl32(v)| = min(r, 2^29 - r) 2^(E - 52), with E the
exponent and r the 29 mantissa bits below f32's precision. Checked here
against exact rational arithmetic, including values that round up into the
next binade, exact halves and the ends of the f32 range."""
from fractions import Fraction

import numpy as np


def _bits_error(v):
    b = int(np.array([v], dtype=np.float64).view(np.uint64)[0])
    e = ((b >> 52) & 0x7FF) - 1023
    assert -126 <= e <= 127
    low = b & ((1 << 29) - 1)
    q = min(low, (1 << 29) - low)
    return Fraction(q) * Fraction(2) ** (e - 52)


def _cases():
    rng = np.random.default_rng(11)
    v = [rng.normal(size=4000) * 10.0 ** rng.integers(-37, 38, 4000), rng.uniform(-1, 1, 2000)]
    edge = [1.0 + 2.0 ** -24, 1.0 + 2.0 ** -24 + 2.0 ** -52,  # an exact half, just above it
            2.0 - 2.0 ** -53,                                  # rounds up into the next binade
            1.1754943508222875e-38, -2.0 ** -126,              # the f32 normal minimum
            3.4028234663852886e38, 3.4028235e38 * 0.9999999,   # near the f32 maximum
            0.5 + 2.0 ** -25, 1.0 - 2.0 ** -54, 123456.789, -7.0e-20]
    return np.concatenate(v + [np.array(edge)])


def test_rounding_error_from_bits_is_exact():
    with np.errstate(over="ignore"):
        for v in _cases():
            f = np.float32(v)
            if not np.isfinite(f):
                continue
            e = ((int(np.array([v]).view(np.uint64)[0]) >> 52) & 0x7FF) - 1023
            if not -126 <= e <= 127:
                continue
            assert _bits_error(v) == abs(Fraction(float(v)) - Fraction(float(f))), v
