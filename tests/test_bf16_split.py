"""The exact three-way BF16 split of the sweep's state columns (bf16_split3 in csrc/sweep.cu),
emulated on the CPU with round-to-nearest-even: hi = bf16(x), mid = bf16(x - hi), lo = bf16(x - hi - mid)
(each residual exact in FP32). hi + mid + lo equals the FP32 value exactly for every x with
2^-102 <= |x| < 2^128 (1 - 2^-9), the point above which bf16(x) rounds past the largest finite BF16,
2^128 (1 - 2^-8), to infinity;
below 2^-102 the last residual's rounding to a BF16 subnormal leaves at most 2^-134 -- far below the
state scales (slip-rate and strain-rate residuals are >= 1e-25 here, states <= 1e10)."""
import numpy as np


def _bf16(x: np.ndarray) -> np.ndarray:
    """Round FP32 to BF16 (nearest, ties to even), returned as FP32."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16
    return b.astype(np.uint32).view(np.float32)


def _split3(x):
    x = np.asarray(x, dtype=np.float32)
    hi = _bf16(x)
    r1 = (x - hi).astype(np.float32)
    mid = _bf16(r1)
    r2 = (r1 - mid).astype(np.float32)
    lo = _bf16(r2)
    return hi, mid, lo, r1, r2


def test_split_is_exact_over_the_normal_range():
    rng = np.random.default_rng(0)
    e = rng.integers(-100, 100, 200000)
    x = (rng.uniform(1, 2, e.size) * 2.0 ** e * rng.choice([-1, 1], e.size)).astype(np.float32)
    big = np.float32(2.0 ** 128 * (1 - 2.0 ** -9) * (1 - 2.0 ** -16))  # just under the rounding limit
    x = np.concatenate([x, np.float32([0.0, 1.0, -1.0, 3.0, 1 + 2 ** -23, 2 ** -100, big, -big])])
    hi, mid, lo, r1, r2 = _split3(x)
    # each residual is exact in FP32 (x - hi and r1 - mid are representable)
    assert np.array_equal(r1.astype(np.float64), x.astype(np.float64) - hi.astype(np.float64))
    assert np.array_equal(r2.astype(np.float64), r1.astype(np.float64) - mid.astype(np.float64))
    # the last residual fits BF16, so the three parts sum to x exactly (in exact arithmetic)
    assert np.array_equal(lo, r2)
    total = hi.astype(np.float64) + mid.astype(np.float64) + lo.astype(np.float64)
    assert np.array_equal(total, x.astype(np.float64))
    # and every product with a BF16 matrix entry is exact in FP32: 8 x 8 significand bits
    q = _bf16(rng.standard_normal(x.size).astype(np.float32))
    for part in (hi, mid, lo):
        p32 = (q * part).astype(np.float32)
        finite = np.isfinite(p32) & (np.abs(p32) > np.finfo(np.float32).tiny)
        assert np.array_equal(p32[finite].astype(np.float64), q[finite].astype(np.float64) * part[finite].astype(np.float64))


def test_largest_finite_bf16_is_the_upper_limit():
    top = np.float32(2.0 ** 128 * (1 - 2.0 ** -8))
    assert np.isfinite(_bf16(top)) and _bf16(top) == top
    assert np.isinf(_bf16(np.float32(2.0 ** 128 * (1 - 2.0 ** -9))))  # the halfway point rounds up (ties to even)
    assert np.isinf(_bf16(np.finfo(np.float32).max))


def test_split_below_the_normal_residual_range_is_bounded():
    rng = np.random.default_rng(1)
    x = (rng.uniform(1, 2, 10000) * 2.0 ** rng.integers(-126, -102, 10000)).astype(np.float32)
    hi, mid, lo, _, _ = _split3(x)
    err = np.abs(hi.astype(np.float64) + mid.astype(np.float64) + lo.astype(np.float64) - x.astype(np.float64))
    assert err.max() <= 2.0 ** -134
