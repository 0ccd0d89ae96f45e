"""Hard-edged aperture masks (dLux utils/geometry.py:20-216), host-side setup."""

from __future__ import annotations

import numpy as np

__all__ = ["circle", "spider", "combine", "block_reduce"]


def _np(coords):
    return np.asarray(coords.cpu() if hasattr(coords, "cpu") else coords, np.float64)


def circle(coords, radius, invert=False):
    """1 inside (or outside when invert) a disk of the given radius."""
    c = _np(coords)
    d = np.hypot(c[0], c[1]) - radius
    return (d > 0).astype(float) if invert else (d < 0).astype(float)


def spider(coords, width, angles):
    """0 on each vane: the half-strip |x'| < w/2, y' < 0 in the frame rotated by the angle."""
    c = _np(coords)
    blocked = np.zeros(c.shape[1:], bool)
    for angle in np.atleast_1d(np.asarray(angles, float)):
        t = -np.deg2rad(angle)
        xr = np.cos(t) * c[0] + np.sin(t) * c[1]
        yr = -np.sin(t) * c[0] + np.cos(t) * c[1]
        blocked |= np.maximum(np.abs(xr) - width / 2, yr) < 0
    return (~blocked).astype(float)


def block_reduce(a, n, mean=True):
    """k x k block mean (or sum) of a square array."""
    s = a.shape[0]
    r = a.reshape(s // n, n, s // n, n).sum(axis=(1, 3))
    return r / (n * n) if mean else r


def combine(arrays, oversample=1, use_sum=False):
    arr = np.array(arrays)
    arr = arr.sum(0) if use_sum else arr.prod(0)
    return arr if oversample == 1 else block_reduce(arr, oversample)
