"""Image error metrics.

`mse`, `rmse`, `rrmse` follow Metrics.h:8-68 (the reference's own, never
called there): sums over width*height*3 values; RRMSE is RMSE divided by
(sqrt(sum of squared ground truth) + 1e-2) — not the usual relative MSE.
`relmse` is the relative MSE used for guiding comparisons:
mean((x - r)^2 / (r^2 + eps)); `relmse_robust` leaves out the pixels with
the largest 0.1 % of per-pixel errors (a few fireflies from a sun lobe
otherwise decide the mean).  Sums are accumulated in float64.
"""
from __future__ import annotations

import numpy as np


def _check(test: np.ndarray, gt: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    t = np.asarray(test, np.float64).ravel()
    g = np.asarray(gt, np.float64).ravel()
    if t.shape != g.shape:
        raise ValueError("test image and ground truth differ in size")
    return t, g


def mse(test, gt) -> float:
    t, g = _check(test, gt)
    return float(np.mean((t - g) ** 2))


def rmse(test, gt) -> float:
    return float(np.sqrt(mse(test, gt)))


def rrmse(test, gt) -> float:
    t, g = _check(test, gt)
    return float(np.sqrt(np.mean((t - g) ** 2)) / (np.sqrt(np.sum(g * g)) + 1e-2))


def relmse(test, gt, eps: float = 1e-2) -> float:
    t, g = _check(test, gt)
    return float(np.mean((t - g) ** 2 / (g * g + eps)))


def relmse_robust(test, gt, eps: float = 1e-2, drop: float = 1e-3) -> float:
    """relMSE over (H, W, 3) images without the largest `drop` share of the
    per-pixel errors (channel means)."""
    t = np.asarray(test, np.float64)
    g = np.asarray(gt, np.float64)
    if t.shape != g.shape:
        raise ValueError("test image and ground truth differ in size")
    d = t - g
    e = np.sort((d * d / (g * g + eps)).reshape(-1, t.shape[-1]).mean(axis=1))
    k = max(1, int(len(e) * drop))
    return float(e[:-k].mean())
