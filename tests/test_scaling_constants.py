"""CPU: the force's constant divisions of the FUSED FP32 kernels
(lane_math.cuh div360 / div3: x * Ch + RN(x * Cl), Ch = RN(1/d), Cl =
RN(1/d - Ch), one multiply and one fused multiply-add) give the correctly
rounded FP32 quotient x / d, checked with exact rational arithmetic on seeded
FP32 inputs across binades; the single multiplication by RN(1/d) does not.
The GPU evaluates the same IEEE operations (FMUL and FFMA, round to nearest
even), so it gives the same bits."""
import random
from fractions import Fraction as Fr

import numpy as np

# the hexadecimal constants written in lane_math.cuh
CONSTANTS = {360: (float.fromhex("0x1.6c16c2p-9"), float.fromhex("-0x1.27d27ep-34")),
             3: (float.fromhex("0x1.555556p-2"), float.fromhex("-0x1.555556p-27"))}


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


def test_constants_are_the_rounded_reciprocal_and_its_remainder():
    for d, (ch, cl) in CONSTANTS.items():
        assert np.float32(ch) == rn32(Fr(1, d))
        assert np.float32(cl) == rn32(Fr(1, d) - Fr(ch))


def test_two_term_multiply_is_correctly_rounded():
    rng = random.Random(7)
    for d, (ch, cl) in CONSTANTS.items():
        single_wrong = 0
        for _ in range(3000):
            m = rng.randint(1 << 23, (1 << 24) - 1)
            x = np.float32(rng.choice((-1, 1)) * m * 2.0 ** (rng.randint(-40, 40) - 23))
            X = Fr(float(x))
            exact = rn32(X / d)
            p = rn32(X * Fr(cl))                   # x * Cl, rounded
            q = rn32(X * Fr(ch) + Fr(float(p)))    # fma(x, Ch, p), one rounding
            assert q == exact, (d, float(x))
            single_wrong += rn32(X * Fr(ch)) != exact
        assert single_wrong > 300  # the single multiplication is off in a sizeable share
