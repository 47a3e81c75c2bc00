"""Seeded synthetic field elements.

SplitMix64 (Steele, Lea, Flood 2014) with the given seed; element i takes the
generator outputs 2i (low 64 bits) and 2i+1 (high 64 bits) and uses the
128-bit value directly as Polyval's raw Montgomery-form value, the way
`FromUniformBytes::try_from_uniform_bytes` accepts any 16 bytes
(p3/src/polyval.rs:71-77).
"""
import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(count: int, seed: int = 0, start: int = 0) -> np.ndarray:
    """Outputs start .. start+count-1 of SplitMix64(seed) as uint64."""
    with np.errstate(over="ignore"):
        idx = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def random_elems(n: int, seed: int = 0, start: int = 0) -> np.ndarray:
    """n field elements as a (n, 16) uint8 array (raw LE u128)."""
    words = splitmix64(2 * n, seed, 2 * start)
    return words.view(np.uint8).reshape(n, 16).copy()
