"""Detector layers (dLux layers/detector_layers.py:22-293)."""

from __future__ import annotations

import torch

from .optical_layers import BaseLayer, as_array

__all__ = ["DetectorLayer", "ApplyPixelResponse", "Downsample", "AddConstant",
           "ApplySaturation", "ApplyJitter"]


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


def gaussian_kernel(std, npixels, extent=5.0):
    """Normalised separable Gaussian on linspace(-extent, extent, npixels) per axis
    (utils/math.py:20-69), as a differentiable torch tensor."""
    std = std if isinstance(std, torch.Tensor) else torch.as_tensor(float(std),
                                                                   dtype=torch.float64)
    x = torch.linspace(-extent, extent, int(npixels), dtype=torch.float64, device=std.device)
    g = torch.exp(-0.5 * (x / std) ** 2) / (std * (2 * torch.pi) ** 0.5)
    k = g[None, :] * g[:, None]
    return k / k.sum()


class ApplyJitter(DetectorLayer):
    """Convolution with a Gaussian of standard deviation ``sigma`` (layers/detector_layers.py:
    134-199): the kernel is built on kernel_size * oversample points and summed down by
    ``oversample``; the convolution runs on the device."""

    def __init__(self, sigma, kernel_size=9, oversample=3):
        self.kernel_size = int(kernel_size)
        if self.kernel_size <= 0:
            raise ValueError("kernel_size must be greater than 0.")
        self.sigma = sigma if isinstance(sigma, torch.Tensor) else torch.as_tensor(
            float(sigma), dtype=torch.float64)
        self.oversample = int(oversample)

    @property
    def kernel(self):
        k = gaussian_kernel(self.sigma, self.kernel_size * self.oversample)
        n, o = self.kernel_size, self.oversample
        return k.reshape(n, o, n, o).sum(dim=(1, 3)).to(torch.float32)

    def __call__(self, psf):
        return psf.convolve(self.kernel)


class ApplySaturation(DetectorLayer):
    """min(psf, threshold) (detector_layers.py:202-231)."""

    def __init__(self, threshold):
        self.threshold = float(threshold)

    def __call__(self, psf):
        return psf.set(data=torch.clamp(psf.data, max=self.threshold))
