"""Coordinate specification (dLux coordinates.py:74-157)."""

from __future__ import annotations

import torch

from .base import Base

__all__ = ["CoordSpec", "PadSpec"]


class CoordSpec(Base):
    """Sampling of one axis: n pixels of size d centred on c."""

    def __init__(self, n=None, d=None, c=0.0):
        self.n = n
        self.d = None if d is None else float(d)
        self.c = None if c is None else float(c)

    @property
    def xs(self):
        if self.d is None:
            raise ValueError("d must be specified to calculate coordinates.")
        return self.c + (torch.arange(self.n, dtype=torch.float64) - (self.n - 1) / 2) * self.d

    @property
    def fov(self):
        if self.d is None:
            raise ValueError("d must be specified to calculate FOV.")
        return self.n * self.d

    @property
    def extent(self):
        if self.d is None:
            raise ValueError("d must be specified to calculate extent.")
        return self.c - (self.n / 2) * self.d, self.c + (self.n / 2) * self.d


class PadSpec(Base):
    """Sampling given as integer padding and cropping factors relative to an
    input grid (dLux coordinates.py:34-72): the padded grid has n * pad pixels,
    the cropped one (n * pad) // crop, centred on c."""

    def __init__(self, pad=1, crop=1, c=0.0):
        self.pad = int(pad)
        self.crop = int(crop)
        self.c = float(c)
