"""Propagator layers (dLux layers/propagators.py:11-217)."""

from __future__ import annotations

from ..coordinates import CoordSpec
from .optical_layers import OpticalLayer

__all__ = ["MFT", "FFT"]


class Propagator(OpticalLayer):
    def __init__(self, focal_length=None, inverse=False):
        self.focal_length = None if focal_length is None else float(focal_length)
        self.inverse = bool(inverse)


class FFT(Propagator):
    """Padded FFT propagation, centred output, then crop (propagators.py:57-142)."""

    def __init__(self, focal_length=None, inverse=False, pad=1, crop=1, center=True):
        super().__init__(focal_length=focal_length, inverse=inverse)
        self.pad = int(pad)
        self.crop = int(crop)
        self.center = bool(center)

    def __call__(self, wavefront):
        spec = CoordSpec(c=0.0) if self.center else None
        size_out = wavefront.npixels * self.pad // self.crop
        return wavefront.propagate_FFT(pad=self.pad, focal_length=self.focal_length,
                                       inverse=self.inverse, spec_out=spec).resize(size_out)


class MFT(Propagator):
    """MFT propagation to npixels at pixel_scale (propagators.py:145-217)."""

    def __init__(self, npixels, pixel_scale, focal_length=None, inverse=False):
        super().__init__(focal_length=focal_length, inverse=inverse)
        self.pixel_scale = float(pixel_scale)
        self.npixels = int(npixels)

    def __call__(self, wavefront):
        return wavefront.propagate(npixels=self.npixels, pixel_scale=self.pixel_scale,
                                   focal_length=self.focal_length, inverse=self.inverse)
