"""Point-spread-function container (dLux psfs.py:14-274)."""

from __future__ import annotations

import torch

from . import autograd
from .base import Base
from .utils import array_ops

__all__ = ["PSF"]


class PSF(Base):
    """Intensity image and its pixel scale."""

    def __init__(self, data, pixel_scale):
        self.data = data if isinstance(data, torch.Tensor) else torch.as_tensor(
            data, dtype=torch.float32, device="cuda" if torch.cuda.is_available() else "cpu")
        self.pixel_scale = pixel_scale

    @property
    def npixels(self):
        return self.data.shape[-1]

    @property
    def ndim(self):
        ps = self.pixel_scale
        return ps.dim() if isinstance(ps, torch.Tensor) else 0

    def downsample(self, n):
        """k x k block sum (psfs.py:74-91) on the device."""
        return self.set(data=autograd.downsample(self.data, n, mean=False),
                        pixel_scale=self.pixel_scale * n)

    def convolve(self, other, method="auto"):
        """Convolution with ``other``, mode "same" (psfs.py:93-110), on the device."""
        if method not in ("auto", "direct", "fft"):
            raise ValueError("method must be 'auto', 'direct' or 'fft'.")
        return self.set(data=autograd.conv2d_same(self.data, other))

    def resize(self, npixels):
        return self.set(data=array_ops.resize(self.data, npixels))

    def flip(self, axis):
        return self.set(data=torch.flip(self.data, dims=(axis,) if isinstance(axis, int) else axis))

    def _op(self, other, op):
        if other is None:
            return self
        if isinstance(other, PSF):
            other = other.data
        if not isinstance(other, (torch.Tensor, float, int, complex)):
            raise TypeError(f"Unsupported type for {op}: {type(other)}. Must be an array, PSF, "
                            "or None.")
        if op == "multiply" and isinstance(other, torch.Tensor) and other.shape == self.data.shape:
            # pixel response: the detector kernel with k = 1
            return self.set(data=autograd.downsample(self.data, 1, False, other.to(torch.float32)))
        if op == "add":
            return self.set(data=self.data + other)
        if op == "subtract":
            return self.set(data=self.data - other)
        if op == "multiply":
            return self.set(data=self.data * other)
        if op == "divide":
            return self.set(data=self.data / other)
        raise ValueError(f"Unsupported operation '{op}'.")

    def __add__(self, o): return self._op(o, "add")
    def __sub__(self, o): return self._op(o, "subtract")
    def __mul__(self, o): return self._op(o, "multiply")
    def __truediv__(self, o): return self._op(o, "divide")
    __iadd__ = __add__
    __isub__ = __sub__
    __imul__ = __mul__
    __itruediv__ = __truediv__
