"""Seeded synthetic initial conditions.

The reference draws its initial fields from Go's math/rand
(examples/cahnHilliard/main.go:20-23), a stream that cannot be reproduced
without Go.  This project's inputs come from SplitMix64 instead: draw i of
seed s is splitmix64 applied to s + (i+1) * 0x9E3779B97F4A7C15, mapped to a
double in [0, 1) by its top 53 bits.  Both the device tests and the CPU
oracle read the same arrays.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64_uniform(seed: int, n: int) -> np.ndarray:
    """n doubles in [0, 1) from SplitMix64 seeded with `seed`."""
    with np.errstate(over="ignore"):
        i = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform_field(seed: int, n: int, center: float, half_width: float) -> np.ndarray:
    """center + U(-half_width, half_width), i.i.d. per cell."""
    return center + half_width * (2.0 * splitmix64_uniform(seed, n) - 1.0)


def splitmix64_ints(seed: int, n: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        i = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))
