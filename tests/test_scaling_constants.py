"""CPU: the constant divisions of the FUSED kernels (lane_math.cuh div3 / div36
/ div360: x * Ch + RN(x * Cl), Ch = RN(1/d), Cl = RN(1/d - Ch), one multiply
and one fused multiply-add) give the correctly rounded FP32 quotient x / d.
Checked with exact integer arithmetic over a sweep of one binade's mantissas
(the rounding decisions scale with the binade for every |x| >= 2^-93, where
x * Cl stays normal) and with exact rationals on seeded values across
binades; the single multiplication by RN(1/d) is wrong for a sizeable share.
The GPU evaluates the same IEEE operations (FMUL and FFMA, round to nearest
even), so it gives the same bits."""
import random
from fractions import Fraction as Fr

import numpy as np

# the hexadecimal constants written in lane_math.cuh: d -> (Ch, Cl)
CONSTANTS = {3: (float.fromhex("0x1.555556p-2"), float.fromhex("-0x1.555556p-27")),
             36: (float.fromhex("0x1.c71c72p-6"), float.fromhex("-0x1.c71c72p-33")),
             360: (float.fromhex("0x1.6c16c2p-9"), float.fromhex("-0x1.27d27ep-34"))}


def rn32(v: Fr) -> np.float32:
    """The FP32 value nearest to the rational v (ties to even), normal range."""
    c = np.float32(float(v))
    best = None
    for cand in (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))):
        err = abs(Fr(float(cand)) - v)
        even = (int(np.float32(cand).view(np.int32)) & 1) == 0
        if best is None or err < best[0] or (err == best[0] and even):
            best = (err, np.float32(cand))
    return best[1]


def _int_form(f: float):
    """f = m * 2^e with |m| a 24-bit integer."""
    m, e = np.frexp(f)
    return int(m * (1 << 24)), int(e) - 24


def _round24(num: int, exp: int, sticky: bool = False):
    """num * 2^exp (num > 0) rounded to a 24-bit mantissa, ties to even;
    sticky: nonzero bits below num."""
    s = num.bit_length() - 24
    if s <= 0:
        return num << -s, exp + s
    q, r, half = num >> s, num & ((1 << s) - 1), 1 << (s - 1)
    if r > half or (r == half and (sticky or (q & 1))):
        q += 1
    if q == 1 << 24:
        q, s = q >> 1, s + 1
    return q, exp + s


def test_constants_are_the_rounded_reciprocal_and_its_remainder():
    for d, (ch, cl) in CONSTANTS.items():
        assert np.float32(ch) == rn32(Fr(1, d))
        assert np.float32(cl) == rn32(Fr(1, d) - Fr(ch))


def test_binade_sweep_is_correctly_rounded():
    """x = M 2^-23 for every 16th mantissa M of [2^23, 2^24), exact integers."""
    K = 64
    for d, (ch, cl) in CONSTANTS.items():
        mc, ec = _int_form(ch)
        ml, el = _int_form(cl)
        assert mc > 0 and ml < 0
        for M in range(1 << 23, 1 << 24, 16):
            pm, pe = _round24(M * -ml, el - 23)          # |x Cl| rounded
            e0 = min(ec - 23, pe)
            s = (M * mc << (ec - 23 - e0)) - (pm << (pe - e0))  # x Ch + RN(x Cl), exact
            got = _round24(s, e0)
            qq, rem = divmod(M << K, d)                  # x / d, exact quotient and sticky bit
            want = _round24(qq, -23 - K, rem != 0)
            assert got == want, (d, M)


def test_seeded_values_across_binades():
    rng = random.Random(7)
    for d, (ch, cl) in CONSTANTS.items():
        single_wrong = 0
        for _ in range(1500):
            m = rng.randint(1 << 23, (1 << 24) - 1)
            x = np.float32(rng.choice((-1, 1)) * m * 2.0 ** (rng.randint(-40, 40) - 23))
            X = Fr(float(x))
            exact = rn32(X / d)
            p = rn32(X * Fr(cl))                   # x * Cl, rounded
            q = rn32(X * Fr(ch) + Fr(float(p)))    # fma(x, Ch, p), one rounding
            assert q == exact, (d, float(x))
            single_wrong += rn32(X * Fr(ch)) != exact
        assert single_wrong > 100  # the single multiplication is off in a sizeable share
