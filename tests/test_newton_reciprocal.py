"""The ensemble kernel's FP64 reciprocal (ens_rcp in csrc/ensemble.cu): the correctly rounded FP32
reciprocal of x rounded to FP32, refined by two Newton-Raphson steps r <- fma(r, fma(-x, r, 1), r).
Replayed here with exactly rounded FMAs (rational arithmetic, then one rounding to FP64, as the
hardware FMA does) over 60 decades of both signs: the result is within 2^-52 of 1/x, about one
unit in the last place -- the accuracy the friction quotient, the error-norm ratios and the Adams
coefficients it replaces FP64 divisions in need."""
from fractions import Fraction

import numpy as np


def _fma(a: float, b: float, c: float) -> float:
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _rcp(x: float) -> float:
    ax = abs(x)
    if not (1e-36 < ax < 1e36):
        return 1.0 / x
    r = float(np.float32(1.0) / np.float32(x))
    r = _fma(r, _fma(-x, r, 1.0), r)
    return _fma(r, _fma(-x, r, 1.0), r)


def test_two_newton_steps_reach_double_precision():
    rng = np.random.default_rng(7)
    xs = 10.0 ** rng.uniform(-30, 30, 1500) * rng.choice([-1.0, 1.0], 1500)
    xs = np.concatenate([xs, [1.0, 3.0, 1e-35, 9.99e35, 0.1, 7.0 / 3.0]])
    worst = 0.0
    for x in xs:
        r = _rcp(float(x))
        err = abs(Fraction(r) * Fraction(float(x)) - 1)
        worst = max(worst, float(err))
    assert worst <= 2.0 ** -52


def test_outside_fp32_range_divides():
    for x in (1e-40, 5e37, -2e300, 1e-300):
        assert _rcp(x) == 1.0 / x
