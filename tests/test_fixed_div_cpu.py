"""The fixed-divisor division of the plane stencil and the FP64 synthesis (lmweather_gb300/csrc/fixed_div.cuh),
restated step for step in Python with exactly rounded FMAs, against IEEE division on the host. The device code
itself is checked bit for bit against CUDA's division by tests/test_plane_gpu.py; this test pins the method (the
two-term reciprocal, the exact acceptance bound, the zero and fallback cases) without a GPU."""
import math
import random
import struct
from fractions import Fraction

ABS = (1 << 63) - 1
MANT = (1 << 52) - 1


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def fma(a, b, c):
    """a * b + c rounded once (Python floats round to nearest even)."""
    if not all(map(math.isfinite, (a, b, c))):
        return a * b + c
    v = Fraction(a) * Fraction(b) + Fraction(c)
    if v == 0:
        return a * b + c  # the sign rules of an exact zero
    try:
        return float(v)
    except OverflowError:
        return math.inf if v > 0 else -math.inf


def reciprocal(y):
    """zh = RN(1/y), zl = RN(1/y - zh); 1 - y zh is exact for zh = RN(1/y)."""
    zh = 1.0 / y
    e = fma(-y, zh, 1.0)
    assert Fraction(e) == 1 - Fraction(y) * Fraction(zh)
    return zh, e / y


def div_fixed(x, y, zh, zl):
    """Returns (quotient, fast path taken)."""
    q = fma(x, zh, x * zl)
    r = fma(-q, y, x)
    bx, by0 = bits(x), bits(y)
    bq, by, br = bits(q) & ABS, by0 & ABS, bits(r) & ABS
    if bx & ABS == 0:
        return from_bits((bx ^ by0) & ~ABS & ((1 << 64) - 1)), True
    eq = bq >> 52
    et = (by >> 52) + eq - 1023 - 53 - (1 if (bq & MANT) == 0 else 0)
    if 1 <= eq <= 2046 and 1 <= et <= 2046 and br < ((et << 52) | (by & MANT)):
        return q, True
    return x / y, False


def test_quotients_are_the_ieee_ones():
    rng = random.Random(5)
    divisors = [5000.0, 2500.0, 2.5e7, 6.25e6, 3.0, 0.1, 1.0 / 3.0, 7.0, -7.5, 6.37122e6, 2.0 ** -1000, 2.0 ** 1000]
    divisors += [rng.uniform(0.5, 2.0) * 2.0 ** rng.randint(-300, 300) for _ in range(8)]
    fast = total = 0
    for y in divisors:
        zh, zl = reciprocal(y)
        xs = [rng.choice((-1.0, 1.0)) * 10.0 ** rng.uniform(-12, 6) for _ in range(600)]
        xs += [rng.uniform(-1, 1) * 2.0 ** rng.randint(-1070, 1020) for _ in range(200)]
        xs += [float(k) * y for k in range(-20, 21)]
        xs += [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, math.inf, -math.inf]
        for x in xs:
            q, f = div_fixed(x, y, zh, zl)
            try:
                want = x / y
            except ZeroDivisionError:
                continue
            assert bits(q) == bits(want), (x, y, q, want)
            fast += f
            total += 1
    assert fast >= 0.9 * total


def test_stencil_like_dividends_take_the_fast_path():
    rng = random.Random(6)
    for y in (5000.0, 2.5e7):
        zh, zl = reciprocal(y)
        n = 0
        for _ in range(2000):
            x = rng.choice((-1.0, 1.0)) * 10.0 ** rng.uniform(-12, 6)
            q, f = div_fixed(x, y, zh, zl)
            assert bits(q) == bits(x / y)
            n += f
        assert n == 2000


def test_nan_dividend_falls_back():
    zh, zl = reciprocal(5000.0)
    q, f = div_fixed(math.nan, 5000.0, zh, zl)
    assert math.isnan(q) and not f
