"""Detector layers (dLux layers/detector_layers.py:22-293)."""

from __future__ import annotations

import torch

from .optical_layers import BaseLayer, as_array

__all__ = ["DetectorLayer", "ApplyPixelResponse", "Downsample", "AddConstant",
           "ApplySaturation"]


class DetectorLayer(BaseLayer):
    """Base class of layers acting on a PSF."""


class ApplyPixelResponse(DetectorLayer):
    """psf * pixel_response (detector_layers.py:100-131)."""

    def __init__(self, pixel_response):
        self.pixel_response = as_array(pixel_response)
        if self.pixel_response.dim() != 2:
            raise ValueError("pixel_response must be a 2d array.")

    def __call__(self, psf):
        return psf * self.pixel_response


class Downsample(DetectorLayer):
    """k x k sum downsample (detector_layers.py:262-293)."""

    def __init__(self, kernel_size):
        self.kernel_size = int(kernel_size)
        if self.kernel_size <= 0:
            raise ValueError("kernel_size must be greater than 0.")

    def __call__(self, psf):
        return psf.downsample(self.kernel_size)


class AddConstant(DetectorLayer):
    """psf + value (detector_layers.py:234-259)."""

    def __init__(self, value):
        self.value = float(value)

    def __call__(self, psf):
        return psf + self.value


class ApplySaturation(DetectorLayer):
    """min(psf, threshold) (detector_layers.py:202-231)."""

    def __init__(self, threshold):
        self.threshold = float(threshold)

    def __call__(self, psf):
        return psf.set(data=torch.clamp(psf.data, max=self.threshold))
