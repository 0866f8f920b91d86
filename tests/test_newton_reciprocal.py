"""The ensemble kernel's FP64 reciprocal (ens_rcp_in_range in csrc/ensemble.cu): the correctly rounded FP32
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


def _rcp_plain(x: float) -> float:
    """The same steps in plain float64 (for arguments whose seed is infinite or zero)."""
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        r = float(np.float32(1.0) / np.float32(x))
        r = r * (-x * r + 1.0) + r
        return r * (-x * r + 1.0) + r


def test_outside_fp32_range():
    # below FP32's normal range the seed overflows: not finite, so the step control rejects the stage
    for x in (1e-40, -1e-300):
        assert not np.isfinite(_rcp_plain(x))
    # above it the seed underflows and the result is zero; the kernel's arguments stay far below
    for x in (1e39, -2e300):
        assert _rcp_plain(x) == 0.0
