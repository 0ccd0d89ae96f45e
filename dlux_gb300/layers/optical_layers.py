"""Optical layers (dLux layers/optical_layers.py:22-371).

Each layer keeps dLux's ``__call__(wavefront) -> wavefront`` contract. Layers
that only multiply the field by a wavelength-independent amplitude, OPD or
phase also describe themselves to ``PupilAccumulator`` so that a layered
optical system can run the whole stack as one fused polychromatic launch.
"""

from __future__ import annotations

import torch

from .. import autograd, kernels
from ..base import Base

__all__ = ["BaseLayer", "OpticalLayer", "TransmissiveLayer", "AberratedLayer", "BasisLayer",
           "Tilt", "Normalise", "PupilAccumulator", "NotFusable"]


def _dev():
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


def as_array(value, dtype=torch.float32):
    """Keep tensors (and their autograd graph); move other arrays to the device."""
    if value is None or hasattr(value, "evaluate"):
        return value
    if isinstance(value, torch.Tensor):
        return value if value.device.type == _dev().type else value.to(_dev())
    return torch.as_tensor(value, dtype=dtype, device=_dev())


class NotFusable(Exception):
    """Raised by a layer that cannot be folded into the fused pupil description."""


class PupilAccumulator:
    """Wavelength-independent description of a pupil-plane layer stack.

    E = A exp(i (2 pi (opd + tilt . xy) / lambda + phase)) with
    A = prod(post) * prod(pre) / sqrt(sum prod(pre)^2) after a normalise, or
    A = prod(pre) / N^2 without one (the 1/N^2 initial field, wavefronts.py:111).
    """

    def __init__(self, npixels, wavefront=None, pixel_scale=None):
        self.n = npixels
        self.wavefront = wavefront
        self.pixel_scale = (pixel_scale if pixel_scale is not None else
                            (wavefront.pixel_scale if wavefront is not None else None))
        self.pre, self.post = [], []
        self.normalised = False
        self.opd = None
        self.phase = None
        self.opd_static = []
        self.phase_static = []
        self.tilt = torch.zeros(2, dtype=torch.float64)  # radians; may carry a gradient
        self.amp_scale = None  # set by fields() when it computed the normalisation

    def amplitude(self, t):
        if t is None:
            return
        (self.post if self.normalised else self.pre).append(t)

    def normalise(self):
        self.pre = self.pre + self.post
        self.post = []
        self.normalised = True

    def add_opd(self, opd):
        if opd is not None:
            self.opd_static.append(opd)

    def add_phase(self, phase):
        if phase is not None:
            self.phase_static.append(phase)

    def add_basis(self, basis, coeffs, effect):
        if effect == "opd":
            self.opd = ("basis", basis, coeffs, self.opd)
        elif effect == "phase":
            self.phase = ("basis", basis, coeffs, self.phase)
        else:
            self.amplitude(("one_plus_basis", basis, coeffs))

    # ---- materialise on the device ----
    @staticmethod
    def _realise(t):
        if isinstance(t, tuple) and t[0] == "one_plus_basis":
            _, basis, coeffs = t
            ones = torch.ones(basis.shape[-2:], dtype=torch.float32, device=basis.device)
            return autograd.eval_basis(basis, coeffs, ones)
        return t

    def _chain(self, node, static):
        base = None
        for s in static:
            base = s if base is None else base + s
        items = []
        while node is not None:
            items.append(node)
            node = node[3]
        for _, basis, coeffs, _ in reversed(items):
            base = autograd.eval_basis(basis, coeffs.reshape(basis.shape[: coeffs.dim()]), base)
        return base

    def fields(self):
        """(amp, normalise_flag, opd, phase) tensors for the fused kernel."""
        pre = [self._realise(t) for t in self.pre]
        post = [self._realise(t) for t in self.post]
        amp = None
        for t in pre:
            amp = t if amp is None else amp * t
        flag = False
        if self.normalised:
            if post:
                if amp is None:
                    amp = torch.ones((self.n, self.n), dtype=torch.float32, device=_dev())
                amp = amp * torch.rsqrt((amp * amp).sum())
                for t in post:
                    amp = amp * t
            else:
                if amp is None:
                    amp = torch.ones((self.n, self.n), dtype=torch.float32, device=_dev())
                flag = True
        else:
            amp = (torch.full((self.n, self.n), 1.0 / self.n ** 2, device=_dev())
                   if amp is None else amp * (1.0 / self.n ** 2))
        # The normalisation depends on the amplitude alone: on the GPU it runs on
        # a side stream while the OPD and phase are evaluated.
        fork = (kernels.AmpNormFork(amp.detach())
                if flag and amp.is_cuda and (self.opd is not None or self.phase is not None)
                else None)
        try:
            opd = self._chain(self.opd, self.opd_static)
            phase = self._chain(self.phase, self.phase_static)
        finally:
            # joined on every path, so the side stream's write to the scale
            # is ordered before anything that reuses its memory
            self.amp_scale = fork.join() if fork is not None else None
        return amp, flag, opd, phase


class BaseLayer(Base):
    def __call__(self, target):  # pragma: no cover - abstract
        raise NotImplementedError

    def apply(self, target):
        return self(target)

    @staticmethod
    def resolve(value, **kwargs):
        if hasattr(value, "evaluate"):
            return value.evaluate(**kwargs)
        return value


class OpticalLayer(BaseLayer):
    """Base class of layers acting on a Wavefront."""

    def fuse(self, acc: PupilAccumulator) -> None:
        raise NotFusable(type(self).__name__)


class TransmissiveLayer(OpticalLayer):
    """wavefront *= transmission, optionally normalised (optical_layers.py:144-186)."""

    def __init__(self, transmission=None, normalise=False, **kwargs):
        self.transmission = as_array(transmission)
        self.normalise = bool(normalise)
        super().__init__(**kwargs)

    def __call__(self, wavefront):
        t = self.resolve(self.transmission, wavefront=wavefront)
        wavefront *= t
        if self.normalise:
            wavefront = wavefront.normalise()
        return wavefront

    def fuse(self, acc):
        acc.amplitude(self.resolve(self.transmission, wavefront=acc.wavefront))
        if self.normalise:
            acc.normalise()


class AberratedLayer(OpticalLayer):
    """wavefront.add_opd(opd).add_phase(phase) (optical_layers.py:189-236)."""

    def __init__(self, opd=None, phase=None, **kwargs):
        self.opd = as_array(opd)
        self.phase = as_array(phase)
        if isinstance(self.opd, torch.Tensor) and isinstance(self.phase, torch.Tensor):
            if self.opd.shape != self.phase.shape:
                raise ValueError("opd and phase must have the same shape. Got shapes "
                                 f"{tuple(self.opd.shape)} and {tuple(self.phase.shape)}.")
        super().__init__(**kwargs)

    def __call__(self, wavefront):
        wavefront = wavefront.add_opd(self.resolve(self.opd, wavefront=wavefront))
        return wavefront.add_phase(self.resolve(self.phase, wavefront=wavefront))

    def fuse(self, acc):
        acc.add_opd(self.resolve(self.opd, wavefront=acc.wavefront))
        acc.add_phase(self.resolve(self.phase, wavefront=acc.wavefront))


class BasisLayer(OpticalLayer):
    """OPD / phase / amplitude from basis . coefficients (optical_layers.py:239-327)."""

    def __init__(self, basis=None, coefficients=None, effect="opd", coefficient_shape=None,
                 **kwargs):
        super().__init__(**kwargs)
        if basis is not None:
            basis = as_array(basis)
            if coefficients is None:
                if coefficient_shape is None:
                    coefficient_shape = tuple(basis.shape[:-2])
                coefficients = torch.zeros(coefficient_shape, device=basis.device)
            else:
                coefficients = as_array(coefficients)
                coefficient_shape = tuple(coefficients.shape)
            if tuple(basis.shape[: len(coefficient_shape)]) != tuple(coefficient_shape):
                raise ValueError("The coefficient shape must match the leading basis dimensions.")
        self.basis = basis
        self.coefficients = coefficients
        if effect not in ("opd", "phase", "amplitude"):
            raise ValueError("effect must be 'opd', 'phase', or 'amplitude'.")
        self.effect = effect

    def eval_basis(self):
        return autograd.eval_basis(self.basis, self.coefficients)

    def __call__(self, wavefront):
        output = self.eval_basis()
        if self.effect == "phase":
            return wavefront.add_phase(output)
        if self.effect == "opd":
            return wavefront.add_opd(output)
        wavefront *= 1 + output
        return wavefront

    def fuse(self, acc):
        acc.add_basis(self.basis, self.coefficients, self.effect)


class Tilt(OpticalLayer):
    """Tilt by (x, y) radians (optical_layers.py:330-359)."""

    def __init__(self, angles):
        a = angles if isinstance(angles, torch.Tensor) else torch.as_tensor(angles,
                                                                             dtype=torch.float64)
        if a.shape != (2,):
            raise ValueError("angles must be a 1d array of shape (2,).")
        self.angles = a

    def __call__(self, wavefront):
        return wavefront.tilt(self.angles)

    def fuse(self, acc):
        a = self.angles.to(torch.float64)
        acc.tilt = acc.tilt.to(a.device) + a


class Normalise(OpticalLayer):
    """Normalise to unit power (optical_layers.py:362-371)."""

    def __call__(self, wavefront):
        return wavefront.normalise()

    def fuse(self, acc):
        acc.normalise()
