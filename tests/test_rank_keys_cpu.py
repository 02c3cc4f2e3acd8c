"""The top-2 pass's keys (fk_tc.cu rank_quad), in exact rationals. Scores lie
in (1.005, 1.995) 2^E (BIG = 1.5 2^E and 2.02 span < 2^E, fk_mixed.cu
prep_aug_kernel); with cgrid = 3 2^(E+6) and ulp = 2^(E-23), the key of a
score T in column code q (0..127) is fma(ulp, q, (T + cgrid) - cgrid), each
step rounded to nearest f32. Checked: (T + cgrid) - cgrid is T rounded to a
multiple of 128 ulp (within 64 ulp), the fma adds q ulp exactly, so keys
are distinct per (grid value, code), within 192 ulp of their scores, and
their order is the order of (grid value, code)."""
from fractions import Fraction

import numpy as np
from exact32 import f32, round32


def _key(t, q, cgrid, ulp):
    g = round32(round32(t + cgrid) - cgrid)
    return round32(ulp * q + g), g


def test_keys_round_to_the_grid_and_carry_the_code():
    rng = np.random.default_rng(31)
    for e in (-30, -4, 0, 9, 25, 60):
        ulp = Fraction(2) ** (e - 23)
        cgrid = 3 * Fraction(2) ** (e + 6)
        assert f32(float(cgrid)) == cgrid and f32(float(ulp)) == ulp
        lo = float(Fraction(2) ** e)
        for _ in range(400):
            t = f32(lo * (1.005 + 0.99 * rng.random()))
            q = int(rng.integers(0, 128))
            k, g = _key(t, q, cgrid, ulp)
            assert g % (128 * ulp) == 0 and abs(g - t) <= 64 * ulp
            assert k == g + q * ulp  # the code lands exactly in the freed bits
            assert abs(k - t) < 192 * ulp


def test_key_order_is_grid_then_code():
    rng = np.random.default_rng(32)
    e = 11
    ulp = Fraction(2) ** (e - 23)
    cgrid = 3 * Fraction(2) ** (e + 6)
    lo = float(Fraction(2) ** e)
    for _ in range(300):
        a = f32(lo * (1.005 + 0.99 * rng.random()))
        b = a + ulp * int(rng.integers(-300, 300))  # near neighbours, across grid boundaries
        qa, qb = (int(v) for v in rng.integers(0, 128, 2))
        ka, ga = _key(a, qa, cgrid, ulp)
        kb, gb = _key(b, qb, cgrid, ulp)
        assert (ka > kb) == ((ga, qa) > (gb, qb))
        assert (ka == kb) == ((ga, qa) == (gb, qb))
