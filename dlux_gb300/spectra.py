"""Spectra (dLux spectra.py:12-117)."""

from __future__ import annotations

import torch

from .base import Base

__all__ = ["BaseSpectrum", "Spectrum"]


def _dev():
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


class BaseSpectrum(Base):
    pass


class Spectrum(BaseSpectrum):
    """Wavelengths and normalised weights (spectra.py:56-117)."""

    def __init__(self, wavelengths, weights=None):
        self.wavelengths = torch.as_tensor(wavelengths, dtype=torch.float64).reshape(-1) \
            if not isinstance(wavelengths, torch.Tensor) else wavelengths.to(torch.float64)
        if self.wavelengths.dim() != 1:
            raise ValueError("wavelengths must be a 1d array.")
        if weights is None:
            weights = torch.ones(self.wavelengths.shape, device=_dev()) / self.wavelengths.shape[-1]
        w = weights if isinstance(weights, torch.Tensor) else torch.as_tensor(
            weights, dtype=torch.float32, device=_dev())
        w = w.to(_dev()) if w.device.type != _dev().type else w
        if w.dim() == 2:
            self.weights = w / w.sum(-1, keepdim=True)
            if tuple(self.wavelengths.shape) != tuple(w.shape[-1:]):
                raise ValueError("wavelengths and weights must have the same trailing shape.")
        else:
            self.weights = w / w.sum()
            if tuple(self.wavelengths.shape) != tuple(w.shape):
                raise ValueError("wavelengths and weights must have the same shape.")

    def normalise(self):
        if self.weights.dim() == 2:
            return self.set(weights=self.weights / self.weights.sum(-1, keepdim=True))
        return self.set(weights=self.weights / self.weights.sum())
