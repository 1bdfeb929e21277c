"""The kernels decode an RGBA8 channel b as one multiply by RN(1/255) and one
Markstein correction step (q0 = b*r; e = fma(-q0, 255, b); q = fma(e, r, q0))
instead of an IEEE division.  This checks, in exact rational arithmetic with
binary32 round-to-nearest-even, that the result is the correctly rounded
quotient b / 255 for every byte, and that the plain reciprocal multiply is not
(which is why the correction step is there)."""
import math
from fractions import Fraction as F

import numpy as np


def _rn32(x: F) -> F:
    """Round a rational to the nearest binary32 value, ties to even (normal range)."""
    if x == 0:
        return F(0)
    s = -1 if x < 0 else 1
    x = abs(x)
    e = math.floor(math.log2(x)) - 23
    while x / F(2) ** e >= 2 ** 24:
        e += 1
    while x / F(2) ** e < 2 ** 23:
        e -= 1
    m = x / F(2) ** e
    fl = math.floor(m)
    r = m - fl
    if r > F(1, 2) or (r == F(1, 2) and fl % 2 == 1):
        fl += 1
    return s * F(fl) * F(2) ** e


def test_rcp_constant_is_rn_of_one_over_255():
    r = _rn32(F(1, 255))
    assert np.float32(float(r)).view(np.uint32) == 0x3B808081


def test_markstein_decode_is_correctly_rounded_for_every_byte():
    r = _rn32(F(1, 255))
    plain_off = 0
    for b in range(256):
        x = F(b)
        want = _rn32(x / 255)
        q0 = _rn32(x * r)
        e = _rn32(x - 255 * q0)  # fused multiply-add: one rounding
        q = _rn32(e * r + q0)    # fused multiply-add: one rounding
        assert q == want, b
        # and it matches numpy's IEEE binary32 division
        assert np.float32(float(q)) == np.float32(b) / np.float32(255)
        plain_off += q0 != want
    assert plain_off == 126
