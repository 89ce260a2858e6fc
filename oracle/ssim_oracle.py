"""Test infrastructure only (the oracle): a float64 numpy restatement of the SSIM loss
of utils/loss_utils.py:23-58 (gaussian, create_window, _ssim), which
trainer/losses.py:147-196 repeats, and of its gradient with respect to img1. The GPU
kernels are checked against it; nothing outside tests/, the smoke check and bench.py's
baseline arm may import it."""
from __future__ import annotations

import numpy as np

C1, C2 = 0.01 ** 2, 0.03 ** 2


def window_1d(size: int = 11, sigma: float = 1.5) -> np.ndarray:
    """utils/loss_utils.py:23-25 (normalised Gaussian)."""
    x = np.arange(size, dtype=np.float64) - size // 2
    g = np.exp(-x * x / (2.0 * sigma * sigma))
    return g / g.sum()


def _conv(img: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Depthwise 2D correlation with the separable window w (x) w and zero padding
    len(w)//2 — F.conv2d(img, window, padding=5, groups=C) of utils/loss_utils.py:41."""
    r = len(w) // 2
    C, H, W = img.shape
    p = np.zeros((C, H + 2 * r, W + 2 * r))
    p[:, r:r + H, r:r + W] = img
    h = np.zeros((C, H + 2 * r, W))
    for k in range(len(w)):
        h += w[k] * p[:, :, k:k + W]
    out = np.zeros((C, H, W))
    for k in range(len(w)):
        out += w[k] * h[:, k:k + H, :]
    return out


def ssim(img1: np.ndarray, img2: np.ndarray, with_grad: bool = False):
    """Mean SSIM (utils/loss_utils.py:41-56) and, with_grad, d mean / d img1."""
    x = np.asarray(img1, np.float64)
    y = np.asarray(img2, np.float64)
    w = window_1d()
    mu1, mu2 = _conv(x, w), _conv(y, w)
    exx, eyy, exy = _conv(x * x, w), _conv(y * y, w), _conv(x * y, w)
    A = 2 * mu1 * mu2 + C1
    B = 2 * (exy - mu1 * mu2) + C2
    Cc = mu1 ** 2 + mu2 ** 2 + C1
    D = (exx - mu1 ** 2) + (eyy - mu2 ** 2) + C2
    S = A * B / (Cc * D)
    mean = S.mean()
    if not with_grad:
        return mean
    n = S.size
    # dS/dmu1, dS/dexx, dS/dexy per output pixel, times d mean / d S = 1/n
    a = S * (2 * mu2 / A - 2 * mu2 / B - 2 * mu1 / Cc + 2 * mu1 / D) / n
    b = -S / D / n
    c = 2 * S / B / n
    grad = _conv(a, w) + 2 * x * _conv(b, w) + y * _conv(c, w)  # the window is symmetric
    return mean, grad
