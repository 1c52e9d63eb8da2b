"""The table-based sin / cos / atan2 of the FP64 update (tab_sincos,
sin_cosm1, tab_atan2 in csrc/common.cuh), restated step by step in Python
with exactly rounded FMA, checked against mpmath: sin / cos within 1.7e-16
absolute, cos r - 1 within 1e-16 absolute (about an ulp of its own size at
r = 0.8), atan2 within 2 ulp.  This pins
the algorithms and their error bounds; the GPU parity tests pin the
compiled code against the oracle."""
import math
import struct
from fractions import Fraction

import numpy as np
import pytest

from test_trig_table import _table

mpmath = pytest.importorskip("mpmath")


def fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


N, KEY, CS, CM1 = _table()


def trig_round(a):
    b = struct.unpack("<q", struct.pack("<d", a))[0]
    if b < 0 or b >= KEY:
        return -1
    e = (b >> 52) - 1023
    if e < -9:
        return 0
    mant = (b & 0xFFFFFFFFFFFFF) | (1 << 52)
    sh = 45 - e
    return (mant + (1 << (sh - 1))) >> sh


def small(b):
    z = b * b
    return fma(b * z, fma(z, 1 / 120, -1 / 6), b), z * fma(z, 1 / 24, -0.5)


def tab_sincos(a):
    j = trig_round(a)
    assert j >= 0
    b = a - j / 128
    assert Fraction(b) == Fraction(a) - Fraction(j, 128)  # exact reduction
    sb, cb = small(b)
    c, s = CS[j]
    return fma(c, sb, fma(s, cb, s)), fma(-s, sb, fma(c, cb, c))


def sin_cosm1(r):
    j = trig_round(r)
    b = r - j / 128
    sb, cb = small(b)
    c, s = CS[j]
    return fma(c, sb, fma(s, cb, s)), fma(c, cb, fma(-s, sb, CM1[j]))


def tab_atan2(y, x):
    af = np.arctan2(abs(np.float32(y)), np.float32(x)).astype(np.float32)
    j = int(np.rint(af * np.float32(128)))
    c, s = CS[j]
    ay = abs(y)
    d = fma(ay, s, x * c)
    e = fma(-x, s, ay * c)
    r0 = float(np.float32(1) / np.float32(d))
    r = fma(r0, fma(-d, r0, 1.0), r0)
    q = e * r
    eps = fma(r, fma(-d, q, e), q)
    z = eps * eps
    at = fma(eps * z, fma(z, fma(z, -1 / 7, 1 / 5), -1 / 3), eps)
    ang = j / 128 + at
    return -ang if math.copysign(1.0, y) < 0 else ang


def test_sincos_absolute_error():
    mpmath.mp.dps = 40
    rng = np.random.default_rng(0)
    worst = 0.0
    for a in list(rng.random(400) * 2 * np.pi) + [0.0, 2 ** -20, 1 / 256, 1 / 128, math.pi / 2, math.pi, 6.28]:
        s, c = tab_sincos(float(a))
        worst = max(worst, abs(float(mpmath.mpf(s) - mpmath.sin(a))), abs(float(mpmath.mpf(c) - mpmath.cos(a))))
    assert worst < 1.7e-16, worst


def test_sin_cosm1_absolute_error():
    mpmath.mp.dps = 40
    rng = np.random.default_rng(1)
    worst_s = worst_c = 0.0
    for r in list(np.abs(rng.normal(size=300)) * 0.3) + [0.0, 1e-9, 2 ** -9, 0.8]:
        s, cm1 = sin_cosm1(float(r))
        worst_s = max(worst_s, abs(float(mpmath.mpf(s) - mpmath.sin(r))))
        worst_c = max(worst_c, abs(float(mpmath.mpf(cm1) - (mpmath.cos(r) - 1))))
    assert worst_s < 1.7e-16 and worst_c < 1e-16, (worst_s, worst_c)


def test_atan2_ulps():
    mpmath.mp.dps = 40
    rng = np.random.default_rng(2)
    worst = 0.0
    for _ in range(300):
        ang, rad = rng.random() * 2 * np.pi - np.pi, 0.3 + rng.random()
        y, x = float(rad * np.sin(ang)), float(rad * np.cos(ang))
        exact = mpmath.atan2(y, x)
        worst = max(worst, float(abs(mpmath.mpf(tab_atan2(y, x)) - exact) / math.ulp(float(exact))))
    assert worst <= 2.0, worst
    for y, x in [(0.0, 1.0), (-0.0, 1.0), (0.0, -1.0), (-0.0, -1.0), (1.0, 0.0), (-1.0, 0.0), (1e-300, 1.0)]:
        assert tab_atan2(y, x) == math.atan2(y, x)
