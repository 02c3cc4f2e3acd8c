"""The arithmetic of the count and mask passes' marks (fk_tc.cu mask_chunk),
in exact rationals: with every score T in the launch's binade [2^E, 2^(E+1)),
ulp = 2^(E-23), S = 8 / ulp and a threshold th >= 2^(E-2) (lower ones are
sent to -inf), fma.rn.sat.f32(T, S, -th S) is exactly 0 or 1, and 1 exactly
when T > th. Then the two 8-step Horner chains joined by one packed FMA give
the word whose bit b < 16 is column 2(15 - b) and bit b >= 16 column
2(31 - b) + 1 (count_column's layout)."""
from fractions import Fraction

import numpy as np
from exact32 import f32, round32


def _fma_sat(t, s, c):
    r = round32(t * s + c)
    return min(max(r, Fraction(0)), Fraction(1))


def test_marks_are_exact_zero_one_and_strict():
    rng = np.random.default_rng(21)
    for e in (-20, -3, 0, 7, 19, 40):
        ulp = Fraction(2) ** (e - 23)
        s = 8 / ulp
        lo, hi = Fraction(2) ** e, Fraction(2) ** (e + 1)
        for _ in range(300):
            t = f32(float(lo) * (1 + rng.random()))
            assert lo <= t < hi
            kind = rng.integers(0, 4)
            if kind == 0:
                th = t                                   # equal: no mark
            elif kind == 1:
                th = t + ulp * rng.choice([-1, 1])       # one ulp either side
            elif kind == 2:
                th = f32(float(Fraction(2) ** (e - 2)) * (1 + 7 * rng.random()))  # anywhere from 2^(E-2)
            else:
                th = f32(float(t) * (1 + (rng.random() - 0.5) * 1e-6))  # within a few ulp
            if th < Fraction(2) ** (e - 2):
                continue
            c = round32(-th * s)
            assert c == -th * s  # exact: a float times a power of two
            m = _fma_sat(t, s, c)
            assert m in (0, 1)
            assert m == (1 if t > th else 0), (e, float(t), float(th))


def test_marks_at_the_binade_edges():
    # T at the bottom of its binade and thresholds just below it, in the two
    # binades beneath (spacings ulp / 2 and ulp / 4): the smallest nonzero
    # T - th the marks must resolve
    for e in (-5, 0, 12, 33):
        ulp = Fraction(2) ** (e - 23)
        s = 8 / ulp
        t = Fraction(2) ** e
        for th in (t - ulp / 2, t - ulp, Fraction(2) ** (e - 1) - ulp / 4, Fraction(2) ** (e - 2), t, t + ulp):
            assert f32(float(th)) == th
            m = _fma_sat(t, s, round32(-th * s))
            assert m == (1 if t > th else 0), (e, float(th))


def _horner_word(bits):
    """Two 8-step chains over columns 0-15 and 16-31, pairs (2j, 2j+1) packed,
    joined as hi 2^8 + lo; returns e | o << 16."""
    hi_e = hi_o = lo_e = lo_o = 0
    for j in range(8):
        hi_e, hi_o = 2 * hi_e + bits[2 * j], 2 * hi_o + bits[2 * j + 1]
        lo_e, lo_o = 2 * lo_e + bits[2 * j + 16], 2 * lo_o + bits[2 * j + 17]
    e, o = hi_e * 256 + lo_e, hi_o * 256 + lo_o
    assert e < 2 ** 16 and o < 2 ** 16  # exact in f32
    return e | (o << 16)


def _column(b):
    return 2 * (15 - b) if b < 16 else 2 * (31 - b) + 1


def test_mask_word_layout_matches_count_column():
    rng = np.random.default_rng(22)
    for _ in range(500):
        bits = [int(v) for v in rng.integers(0, 2, 32)]
        w = _horner_word(bits)
        for b in range(32):
            assert ((w >> b) & 1) == bits[_column(b)]
