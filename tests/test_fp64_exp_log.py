"""The ensemble kernel's FP64 exp and log (ens_exp, ens_log in csrc/ensemble.cu), replayed step by step
with exactly rounded FMAs (rational arithmetic, one rounding to FP64 per FMA, as the hardware does)
and compared with 40-digit references (decimal): exp within 6 units in the last place over
[-700, 700], log within 6 units (absolute 6 * 2^-53 where |ln x| < 1) over 600 decades. The
friction update they serve is an FP64 computation; a few units in the last place are far inside
the slip-rate tolerances."""
import decimal
import math
from fractions import Fraction

import numpy as np

LN2_HI, LN2_LO, LOG2E = 0.6931471805599453, 2.3190468138462996e-17, 1.4426950408889634
ULP = 2.0 ** -53


def fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def rcp_in_range(x):
    r = float(np.float32(1.0) / np.float32(x))
    r = fma(r, fma(-x, r, 1.0), r)
    return fma(r, fma(-x, r, 1.0), r)


def ens_exp(x):
    if not (-745.2 < x < 709.78):
        return math.exp(x) if x < 709.78 else math.inf
    k = float(np.rint(x * LOG2E))
    r = fma(-k, LN2_HI, x)
    r = fma(-k, LN2_LO, r)
    r2 = r * r
    r4 = r2 * r2
    r8 = r4 * r4
    p0, p1, p2 = fma(1.0, r, 1.0), fma(1.0 / 6, r, 1.0 / 2), fma(1.0 / 120, r, 1.0 / 24)
    p3, p4 = fma(1.0 / 5040, r, 1.0 / 720), fma(1.0 / 362880, r, 1.0 / 40320)
    p5, p6 = fma(1.0 / 39916800, r, 1.0 / 3628800), fma(1.0 / 6227020800.0, r, 1.0 / 479001600)
    q0, q1, q2 = fma(p1, r2, p0), fma(p3, r2, p2), fma(p5, r2, p4)
    s0, s1 = fma(q1, r4, q0), fma(p6, r4, q2)
    e = fma(s1, r8, s0)
    ki = int(k)
    if -1020 <= ki <= 1020:
        return e * 2.0 ** ki
    h = int(ki / 2)
    return e * 2.0 ** h * 2.0 ** (ki - h)


def ens_log(x):
    m, e = math.frexp(x)
    m, e = 2.0 * m, e - 1
    if m > 1.4142135623730951:
        m, e = 0.5 * m, e + 1
    s = (m - 1.0) * rcp_in_range(m + 1.0)
    z = s * s
    z2 = z * z
    z4 = z2 * z2
    z8 = z4 * z4
    p0, p1, p2 = fma(1.0 / 3, z, 1.0), fma(1.0 / 7, z, 1.0 / 5), fma(1.0 / 11, z, 1.0 / 9)
    p3, p4 = fma(1.0 / 15, z, 1.0 / 13), fma(1.0 / 19, z, 1.0 / 17)
    q0, q1, q2 = fma(p1, z2, p0), fma(p3, z2, p2), fma(1.0 / 21, z2, p4)
    t0 = fma(q1, z4, q0)
    P = fma(q2, z8, t0)
    de = float(e)
    return fma(de, LN2_HI, fma(de, LN2_LO, (s + s) * P))


def test_exp_within_a_few_ulp():
    decimal.getcontext().prec = 40
    rng = np.random.default_rng(3)
    worst = 0.0
    for x in np.concatenate([rng.uniform(-700, 700, 1500), rng.uniform(-2, 2, 1000), [0.0, 1.0, -1.0, 0.3465]]):
        ref = decimal.Decimal(float(x)).exp()
        got = decimal.Decimal(ens_exp(float(x)))
        worst = max(worst, float(abs(got - ref) / ref))
    assert worst <= 6 * ULP


def test_log_within_a_few_ulp():
    decimal.getcontext().prec = 40
    rng = np.random.default_rng(4)
    worst = 0.0
    for x in np.concatenate([10.0 ** rng.uniform(-300, 300, 1500), rng.uniform(0.5, 2.0, 1000), [1.0, 2.0, 0.5, 1e10]]):
        ref = decimal.Decimal(float(x)).ln()
        got = decimal.Decimal(ens_log(float(x)))
        err = abs(got - ref) / max(abs(ref), decimal.Decimal(1))
        worst = max(worst, float(err))
    assert worst <= 6 * ULP
