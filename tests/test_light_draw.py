"""The light index of next-event estimation without fp64 arithmetic.

rng.Intn(n) in the reference's CPU integrator takes floor(u * n) of the fp64
product of a 24-bit uniform u = k * 2^-24 and n (capped at n - 1). The device
(`draw_index`, beamcast-gx-v1.0-beta-_gb300/csrc/sampling.cuh) computes
(k * n) >> 24 in integers below n = 2^29, where the fp64 product is exact; this
test checks the two agree on every draw class that matters: random draws, the
largest draw, and the draws on both sides of each index boundary.
"""
import numpy as np


def _fp64(k, n):
    return np.minimum(np.floor(k.astype(np.float64) * 2.0 ** -24 * np.float64(n)).astype(np.int64), n - 1)


def _int(k, n):
    return np.minimum((k.astype(np.uint64) * np.uint64(n)) >> np.uint64(24), np.uint64(n - 1)).astype(np.int64)


def test_integer_light_index_equals_fp64_draw():
    rng = np.random.default_rng(5)
    ns = [1, 2, 3, 7, 64, 1000, 65_537, 2**24 - 1, 2**24 + 3, 123_456_789, 2**29 - 1]
    for n in ns:
        k = rng.integers(0, 2**24, 200_000, dtype=np.int64)
        k = np.concatenate([k, [0, 2**24 - 1]])
        # the draws just below and at each index boundary i * 2^24 / n, for the first indices
        i = np.arange(1, min(n, 4096), dtype=np.int64)
        edge = (i << 24) // n
        k = np.concatenate([k, np.clip(edge - 1, 0, 2**24 - 1), np.clip(edge, 0, 2**24 - 1),
                            np.clip(edge + 1, 0, 2**24 - 1)])
        assert np.array_equal(_int(k, n), _fp64(k, n)), n
