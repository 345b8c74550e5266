"""The kernels divide tile indices by runtime divisors with one multiply-high
(FastDiv in p3g_engine.cuh): q = (2x * (floor((2^31 - 1) / d) + 1)) >> 32
for x, d <= 2^15.  Checked here on a sample of divisors (all of them were
checked once offline)."""
import numpy as np


def test_multiply_high_division_is_exact():
    rng = np.random.default_rng(0)
    x = np.arange(1 << 15, dtype=np.uint64)
    divisors = set(rng.integers(1, (1 << 15) + 1, size=300).tolist()) | {3, 5, 7, 9, 15, 17, 257, 513, 769, 8191}
    for d in sorted(divisors):
        m = np.uint64((0x7FFFFFFF // d) + 1)
        q = ((x << np.uint64(1)) * m) >> np.uint64(32)
        assert np.array_equal(q, x // np.uint64(d)), d
