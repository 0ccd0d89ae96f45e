"""FFT output sampling and phase ramps (dLux utils/fourier.py:14-78)."""

from __future__ import annotations

import math

import torch

__all__ = ["fft_spec", "fft_phase_ramp"]


def fft_spec(npixels_in, pixel_scale_in, wavelength, focal_length=None):
    """Native FFT output pixel scale and centre offset (utils/fourier.py:14-45)."""
    d_out = wavelength / (npixels_in * pixel_scale_in)
    if focal_length is not None:
        d_out = d_out * focal_length
    if npixels_in % 2 != 0:
        return d_out, 0.0
    return d_out, -0.5 * d_out


def fft_phase_ramp(xs, wavelength, shift, focal_length=None, inverse=False):
    """Separable 2-D ramp exp(+-2 pi i xs shift / alpha) (utils/fourier.py:48-78).

    The propagation path folds these ramps into its DFT matrices; this
    function returns the explicit array for callers that want it.
    """
    sign = -1.0 if inverse else 1.0
    alpha = wavelength if focal_length is None else wavelength * focal_length
    x = torch.as_tensor(xs, dtype=torch.float64)
    cyc = sign * x * float(shift) / float(alpha)
    cyc = cyc - torch.round(cyc)
    ramp = torch.polar(torch.ones_like(cyc), 2 * math.pi * cyc)
    return (ramp[None, :] * ramp[:, None]).to(torch.complex64)
