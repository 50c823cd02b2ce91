"""The fast division of the run-time FFT kernels' index arithmetic
(csrc/spe_size_any.cu, fdiv / fdiv_inv): x / d as the high 32 bits of
x * ceil(2^32 / d), restated in numpy and checked exhaustively at the
quotient boundaries (x = q d - 1 and q d) for every divisor 2 <= d < 2^15
and every x < 2^17, the ranges the plans guarantee."""
import numpy as np


def inv_of(d):
    return np.uint64(0xFFFFFFFF // d + 1)


def test_multiply_high_division_is_exact_at_every_boundary():
    limit = 1 << 17
    for d in range(2, 1 << 15):
        q = np.arange(1, (limit - 1) // d + 2, dtype=np.uint64)
        x = np.concatenate([q * np.uint64(d) - np.uint64(1), q * np.uint64(d), np.array([0, limit - 1], np.uint64)])
        x = x[x < limit]
        got = (x * inv_of(d)) >> np.uint64(32)
        assert np.array_equal(got, x // np.uint64(d)), d
