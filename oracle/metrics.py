"""ORACLE (test infrastructure only): the reference's image metrics in numpy.

Restates scripts/eval.py:66-68 (PSNR = -10 log10(MSE) over RGB in [0, 1]) and
scripts/loss_utils.py:17-57 (SSIM: 11x11 Gaussian window, sigma 1.5, zero
padding, per channel, C1 = 0.01^2, C2 = 0.03^2, mean of the map) in float64.
Pinned against the reference's own loss_utils.ssim run with torch on the CPU
(tests/golden/metrics/pairs.npz, written by tests/golden/make_golden.py metrics).
"""
from __future__ import annotations

import math

import numpy as np


def gaussian(window: int = 11, sigma: float = 1.5) -> np.ndarray:
    g = np.array([math.exp(-(x - window // 2) ** 2 / float(2 * sigma ** 2)) for x in range(window)])
    return g / g.sum()


def _filter(img: np.ndarray, g: np.ndarray) -> np.ndarray:
    """Separable zero-padded 'same' correlation of (H, W) with outer(g, g)."""
    r = len(g) // 2
    h, w = img.shape
    p = np.zeros((h + 2 * r, w + 2 * r))
    p[r:r + h, r:r + w] = img
    tmp = sum(g[k] * p[:, k:k + w] for k in range(len(g)))
    return sum(g[k] * tmp[k:k + h, :] for k in range(len(g)))


def to_rgb01(img: np.ndarray) -> np.ndarray:
    """(H, W, 3|4) uint8 -> (3, H, W) float64 in [0, 1] (alpha dropped, eval.py:55-57)."""
    return np.moveaxis(np.asarray(img)[..., :3].astype(np.float64) / 255.0, -1, 0)


def ssim(a: np.ndarray, b: np.ndarray) -> float:
    x, y = to_rgb01(a), to_rgb01(b)
    g = gaussian()
    c1, c2 = 0.01 ** 2, 0.03 ** 2
    vals = []
    for c in range(3):
        mu1, mu2 = _filter(x[c], g), _filter(y[c], g)
        s11 = _filter(x[c] * x[c], g) - mu1 * mu1
        s22 = _filter(y[c] * y[c], g) - mu2 * mu2
        s12 = _filter(x[c] * y[c], g) - mu1 * mu2
        vals.append(((2 * mu1 * mu2 + c1) * (2 * s12 + c2)) / ((mu1 * mu1 + mu2 * mu2 + c1) * (s11 + s22 + c2)))
    return float(np.mean(vals))


def mse(a: np.ndarray, b: np.ndarray) -> float:
    x, y = to_rgb01(a), to_rgb01(b)
    return float(np.mean((x - y) ** 2))


def psnr(a: np.ndarray, b: np.ndarray) -> float:
    m = mse(a, b)
    return math.inf if m == 0 else -10.0 * math.log10(m)
