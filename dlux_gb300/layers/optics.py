"""Composite optics (dLux layers/optics.py:17-175)."""

from __future__ import annotations

import torch

from .optical_layers import AberratedLayer, BasisLayer, TransmissiveLayer

__all__ = ["Optic", "BasisOptic"]


class Optic(TransmissiveLayer, AberratedLayer):
    """Transmission, OPD and phase in one layer (optics.py:17-96)."""

    def __init__(self, transmission=None, opd=None, phase=None, normalise=False):
        super().__init__(transmission=transmission, opd=opd, phase=phase, normalise=normalise)
        if isinstance(self.transmission, torch.Tensor):
            for name in ("opd", "phase"):
                v = getattr(self, name)
                if isinstance(v, torch.Tensor) and v.shape != self.transmission.shape:
                    raise ValueError(f"transmission and {name} must have the same shape. Got "
                                     f"shapes {tuple(self.transmission.shape)} and "
                                     f"{tuple(v.shape)}.")

    def __call__(self, wavefront):
        wavefront *= self.resolve(self.transmission, wavefront=wavefront)
        wavefront = wavefront.add_opd(self.resolve(self.opd, wavefront=wavefront))
        wavefront = wavefront.add_phase(self.resolve(self.phase, wavefront=wavefront))
        if self.normalise:
            wavefront = wavefront.normalise()
        return wavefront

    def fuse(self, acc):
        acc.amplitude(self.resolve(self.transmission, wavefront=acc.wavefront))
        acc.add_opd(self.resolve(self.opd, wavefront=acc.wavefront))
        acc.add_phase(self.resolve(self.phase, wavefront=acc.wavefront))
        if self.normalise:
            acc.normalise()


class BasisOptic(TransmissiveLayer, BasisLayer):
    """Transmission plus a basis-driven OPD/phase/amplitude (optics.py:99-175)."""

    def __init__(self, basis, transmission=None, coefficients=None, normalise=False,
                 effect="opd", coefficient_shape=None):
        super().__init__(transmission=transmission, basis=basis, coefficients=coefficients,
                         normalise=normalise, effect=effect, coefficient_shape=coefficient_shape)

    def __call__(self, wavefront):
        wavefront *= self.resolve(self.transmission, wavefront=wavefront)
        wavefront = BasisLayer.__call__(self, wavefront)
        if self.normalise:
            wavefront = wavefront.normalise()
        return wavefront

    def fuse(self, acc):
        acc.amplitude(self.resolve(self.transmission, wavefront=acc.wavefront))
        acc.add_basis(self.basis, self.coefficients, self.effect)
        if self.normalise:
            acc.normalise()
