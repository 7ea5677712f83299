"""The device code divides by the finite-difference step 1e-8 and by small
grain side counts N with one multiplication and one fma (Brisebarre,
Muller and Raina, IEEE Trans. Computers 53(8), 2004) instead of a
division.  These checks pin the constants in csrc/sevc_device.cuh to
zh = RN(1/y), zl = RN(1/y - zh), re-derive the error bound that makes the
result the correctly rounded quotient, and compare the method, evaluated in
exact rational arithmetic, with Python's correctly rounded division on
random and near-midpoint dividends."""
import math
import os
import random
import re
from fractions import Fraction as F

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "..", "se-grain-growth-gpu_gb300", "csrc", "sevc_device.cuh")


def constants():
    text = open(SRC).read()
    out = {}
    m_hi = re.search(r"#define SEVC_INV_EPS_HI (\S+)", text)
    m_lo = re.search(r"#define SEVC_INV_EPS_LO \((\S+)\)", text)
    out[1e-8] = (float.fromhex(m_hi.group(1)), float.fromhex(m_lo.group(1)))
    for n, hi, lo in re.findall(r"struct InvSplit<(\d+)> \{ static constexpr double hi = (\S+), lo = (\S+); \}", text):
        out[float(n)] = (float.fromhex(hi), float.fromhex(lo))
    return out


def ulp(x):
    _, e = math.frexp(abs(x))
    return math.ldexp(1.0, e - 53)


def fast(x, zh, zl):
    q = float(F(x) * F(zl))             # RN(x * zl)
    return float(F(x) * F(zh) + F(q))    # the fma: one rounding of the exact sum


def test_constants_are_the_split_reciprocal():
    c = constants()
    assert sorted(c) == [1e-8, 3.0, 5.0, 6.0, 7.0, 9.0, 10.0]
    for y, (zh, zl) in c.items():
        assert zh == float(1 / F(y)) and zl == float(1 / F(y) - F(zh)), y


def test_error_bound_below_midpoint_distance():
    """|x zh + RN(x zl) - x/y| / |x/y| <= eps_rel for x in [1, 2) (the
    method is scale invariant in the guarded range).  A quotient of two
    binary64 numbers is at relative distance >= 2^-107 from every rounding
    midpoint (>= 2^-59 when y is an integer <= 10), so eps_rel below that
    makes the fma's rounding the correctly rounded quotient."""
    for y, (zh, zl) in constants().items():
        eps_rel = abs(F(zh) + F(zl) - 1 / F(y)) * F(y) + F(ulp(zl)) * F(y)
        limit = F(1, 2 ** 107) if y < 1 else F(1, 2 ** 59)
        assert eps_rel < limit, (y, math.log2(eps_rel))


def test_matches_correct_rounding_on_samples():
    rnd = random.Random(7)
    for y, (zh, zl) in constants().items():
        for _ in range(3000):
            x = rnd.uniform(1, 2) * 2.0 ** rnd.randint(-800, 800) * rnd.choice((-1, 1))
            assert fast(x, zh, zl) == x / y, (y, x.hex())
        for _ in range(3000):   # dividends whose quotient sits next to a midpoint
            k, e = rnd.randrange(2 ** 52, 2 ** 53), rnd.randint(-700, 700)
            mid = F(2 * k + 1, 2 ** 53) * F(2) ** e
            x0 = float(mid * F(y))
            for x in (x0, math.nextafter(x0, math.inf), math.nextafter(x0, -math.inf)):
                assert fast(x, zh, zl) == x / y, (y, x.hex())
