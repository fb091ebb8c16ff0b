"""Seeded synthetic inputs with the shapes and value distributions of the benchmark workloads.

No public dataset is involved: every input is generated here from numpy's PCG64
(``numpy.random.default_rng(seed)``), Gaussian smoothing is
``scipy.ndimage.gaussian_filter`` in float64 (mode 'reflect', truncate 4.0) and rescaling to
u8 is ``rint((x - min) / (max - min) * 255)``.
"""
from __future__ import annotations

import numpy as np


def uniform_u8(shape, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).integers(0, 256, size=shape, dtype=np.uint8)


def uniform_u16(shape, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).integers(0, 65536, size=shape, dtype=np.uint16)


def normal_f32(shape, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal(size=shape, dtype=np.float32)


def rescale_u8(x: np.ndarray) -> np.ndarray:
    lo, hi = float(x.min()), float(x.max())
    if hi <= lo:
        return np.zeros(x.shape, np.uint8)
    return np.rint((x - lo) / (hi - lo) * 255.0).astype(np.uint8)


def smoothed_noise_u8(shape, seed: int, sigma: float = 4.0) -> np.ndarray:
    """White noise (seed) -> Gaussian(sigma) -> rescaled to the full [0, 255] range."""
    from scipy.ndimage import gaussian_filter
    noise = np.random.default_rng(seed).random(size=shape)
    return rescale_u8(gaussian_filter(noise, sigma, mode="reflect", truncate=4.0))


def leveling_marker(mask: np.ndarray, sigma: float = 16.0) -> np.ndarray:
    """Marker of the leveling workload: the mask Gaussian-smoothed (sigma) in float64, rounded."""
    from scipy.ndimage import gaussian_filter
    m = gaussian_filter(mask.astype(np.float64), sigma, mode="reflect", truncate=4.0)
    return np.clip(np.rint(m), 0, 255).astype(np.uint8)


def ragged_sizes(n: int = 512, lo: int = 64, hi: int = 1024, seed: int = 5):
    """(H, W) of the ragged batch: W then H drawn per image, uniformly in [lo, hi]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        w = int(rng.integers(lo, hi + 1))
        h = int(rng.integers(lo, hi + 1))
        out.append((h, w))
    return out


def ragged_batch(n: int = 512, seed: int = 5, sigma: float = 4.0):
    """The ragged h-maxima batch: per-image seed 5*1000 + i, smoothed noise like smoothed_noise_u8."""
    return [smoothed_noise_u8(hw, seed * 1000 + i, sigma) for i, hw in enumerate(ragged_sizes(n, seed=seed))]
