"""Host (numpy) twin of the device SplitMix64 input generator.

Element i of a stream is mix((seed ^ GAMMA) + (i + 1) * GAMMA) with the step
and mix constants of the reference's test generator
(tests/test_expr_fused_equivalence.rs:96-112), so host and device produce the
same bits for the integer and uniform distributions.
"""
from __future__ import annotations

import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, n: int, start: int = 0) -> np.ndarray:
    with np.errstate(over="ignore"):
        i = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = (np.uint64(seed) ^ GAMMA) + i * GAMMA
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def u01(seed: int, n: int) -> np.ndarray:
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform_pm1(seed: int, n: int) -> np.ndarray:
    return 2.0 * u01(seed, n) - 1.0


def int_range(seed: int, n: int, lo: int = -(1 << 20), width_log2: int = 21) -> np.ndarray:
    """Uniform integers in [lo, lo + 2^width_log2): top bits of each draw."""
    return (splitmix64(seed, n) >> np.uint64(64 - width_log2)).astype(np.int64) + lo
