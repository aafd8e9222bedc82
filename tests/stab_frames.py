"""Seeded synthetic grayscale frames for the stabiliser tests: a smooth random texture (box-blurred
noise, 0..255) and the same texture moved by a whole-pixel translation."""
from __future__ import annotations

import numpy as np


def texture(h: int, w: int, seed: int, blur: int = 3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    img = rng.random((h + 2 * blur, w + 2 * blur))
    for axis in (0, 1):  # box blur of width 2*blur+1, twice
        for _ in range(2):
            c = np.cumsum(np.pad(img, [(1, 0) if a == axis else (0, 0) for a in range(2)]), axis=axis)
            k = 2 * blur + 1
            sl = [slice(None)] * 2
            sl[axis] = slice(k, None)
            lo = [slice(None)] * 2
            lo[axis] = slice(0, -k)
            img = np.pad((c[tuple(sl)] - c[tuple(lo)]) / k, [(blur, blur) if a == axis else (0, 0) for a in range(2)],
                         mode="edge")
    img = img[blur:blur + h, blur:blur + w]
    img = (img - img.min()) / max(float(img.max() - img.min()), 1e-12)
    return (img * 255.0).astype(np.float32)


def moving_pair(h: int, w: int, shift: tuple[int, int], seed: int = 0):
    """(prev, next): next shows prev's content moved by shift = (dx, dy) pixels."""
    dx, dy = shift
    m = max(abs(dx), abs(dy)) + 1
    big = texture(h + 2 * m, w + 2 * m, seed)
    prev = big[m:m + h, m:m + w]
    nxt = big[m - dy:m - dy + h, m - dx:m - dx + w]
    return np.ascontiguousarray(prev), np.ascontiguousarray(nxt)
