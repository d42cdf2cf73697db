"""Deterministic, platform-independent test inputs (splitmix64 in numpy
uint64 arithmetic), so committed fixtures reproduce bit for bit on any
machine and numpy version."""
from __future__ import annotations

import numpy as np

_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix_bytes(seed: int, n: int) -> np.ndarray:
    """n pseudo-random bytes from a seeded splitmix64 stream."""
    words = (n + 7) // 8
    with np.errstate(over="ignore"):
        x = np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + np.arange(1, words + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
        z = x
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z.view(np.uint8)[:n].copy()


def image(seed: int, h: int, w: int, ch: int, pad: int = 0) -> np.ndarray:
    """An h x w (x ch) uint8 view into a buffer with `pad` extra pixels per
    row (a sub-image with a larger stride when pad > 0)."""
    full = splitmix_bytes(seed, h * (w + pad) * ch)
    if ch == 1:
        return full.reshape(h, w + pad)[:, :w]
    return full.reshape(h, w + pad, ch)[:, :w]
