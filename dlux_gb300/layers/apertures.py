"""Dynamic apertures evaluated on the device (layers/apertures.py of dLux).

``CircularAperture``, ``SquareAperture``, ``RectangularAperture`` and
``RegPolyAperture`` are soft-edged masks under an optional ``CoordTransform``
(layers/apertures.py:240-555, utils/geometry.py:49-91, 229-351 and 402-579).
``AberratedAperture`` adds Zernike aberrations defined on any of them
(layers/apertures.py:643-800; polynomials.py:20-51): Zernikes for a circle,
polygon-stretched Zernikes (utils/zernikes.py:318-419) with the shape's side
count otherwise. Both are computed per pixel by ``dlx_aberrated_aperture``,
with no stored basis. The OPD is differentiable with respect to the
coefficients; the aperture geometry is a constant here.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from .. import autograd, kernels
from ..base import Base
from .optical_layers import OpticalLayer

__all__ = ["CoordTransform", "CircularAperture", "SquareAperture", "RectangularAperture",
           "RegPolyAperture", "AberratedAperture"]


class CoordTransform(Base):
    """translation, rotation (clockwise, rad), compression, shear (coordinates.py:240-314)."""

    def __init__(self, translation=None, rotation=None, compression=None, shear=None):
        def vec(v, name):
            if v is None:
                return None
            a = np.asarray(v, dtype=float)
            if a.shape != (2,):
                raise ValueError(f"{name} must have shape (2,).")
            return a
        self.translation = vec(translation, "translation")
        self.compression = vec(compression, "compression")
        self.shear = vec(shear, "shear")
        if rotation is not None and np.asarray(rotation).shape != ():
            raise ValueError("rotation must be a scalar.")
        self.rotation = None if rotation is None else float(rotation)


class DynamicAperture(OpticalLayer):
    """Soft-edged aperture under a CoordTransform (layers/apertures.py:155-237)."""

    def __init__(self, transformation=None, occulting=False, softening=1.0, normalise=False):
        if transformation is not None and not isinstance(transformation, CoordTransform):
            raise TypeError("transformation must be a BaseCoordTransform instance, got "
                            f"{type(transformation).__name__}.")
        if float(softening) <= 0:
            raise ValueError("softening must be greater than 0.")
        self.transformation = transformation
        self.occulting = bool(occulting)
        self.softness = float(softening)
        self.normalise = bool(normalise)

    def _shape(self):  # pragma: no cover - abstract
        raise NotImplementedError

    def desc(self, npixels, pixel_scale):
        t = self.transformation
        return kernels.aperture_desc(npixels, pixel_scale, softening=self.softness,
                                     occulting=self.occulting,
                                     translation=None if t is None else t.translation,
                                     rotation=None if t is None else t.rotation,
                                     compression=None if t is None else t.compression,
                                     shear=None if t is None else t.shear, **self._shape())

    def transmission(self, npixels, pixel_scale):
        trans, _ = kernels.aberrated_aperture(self.desc(npixels, pixel_scale), [], None,
                                              want_opd=False)
        return trans

    def __call__(self, wavefront):
        wavefront *= self.transmission(wavefront.npixels, wavefront.pixel_scale)
        if self.normalise:
            wavefront = wavefront.normalise()
        return wavefront

    def fuse(self, acc):
        acc.amplitude(self.transmission(acc.n, acc.pixel_scale))
        if self.normalise:
            acc.normalise()


class CircularAperture(DynamicAperture):
    """Soft-edged circle of ``radius`` (m) (layers/apertures.py:240-312)."""

    def __init__(self, radius, transformation=None, occulting=False, softening=1.0,
                 normalise=False):
        super().__init__(transformation, occulting, softening, normalise)
        self.radius = float(radius)

    def _shape(self):
        return dict(shape="circle", radius=self.radius)

    @property
    def extent(self):
        return self.radius

    @property
    def nsides(self):
        return 0


class SquareAperture(DynamicAperture):
    """Soft-edged square of side ``width`` (m) (layers/apertures.py:315-388)."""

    def __init__(self, width, transformation=None, occulting=False, softening=1.0,
                 normalise=False):
        super().__init__(transformation, occulting, softening, normalise)
        self.width = float(width)

    def _shape(self):
        return dict(shape="square", radius=0.0, width=self.width)

    @property
    def extent(self):
        return math.sqrt(2) * self.width

    @property
    def nsides(self):
        return 4


class RectangularAperture(DynamicAperture):
    """Soft-edged ``width`` (x) by ``height`` (y) rectangle (layers/apertures.py:391-472)."""

    def __init__(self, height, width, transformation=None, occulting=False, softening=1.0,
                 normalise=False):
        self.height = float(height)
        self.width = float(width)
        super().__init__(transformation, occulting, softening, normalise)

    def _shape(self):
        return dict(shape="rectangle", radius=0.0, width=self.width, height=self.height)

    @property
    def extent(self):
        return math.hypot(self.height / 2.0, self.width / 2.0)

    @property
    def nsides(self):
        return 4


class RegPolyAperture(DynamicAperture):
    """Soft-edged regular polygon of ``nsides`` and circumradius ``rmax``
    (layers/apertures.py:475-555)."""

    def __init__(self, nsides, rmax, transformation=None, occulting=False, softening=1.0,
                 normalise=False):
        super().__init__(transformation, occulting, softening, normalise)
        self._nsides = int(nsides)
        self.rmax = float(rmax)

    def _shape(self):
        return dict(shape="polygon", radius=self.rmax, nsides=self._nsides)

    @property
    def extent(self):
        return self.rmax

    @property
    def nsides(self):
        return self._nsides


class AberratedAperture(OpticalLayer):
    """Zernike aberrations on a dynamic aperture (layers/apertures.py:643-800)."""

    def __init__(self, aperture, noll_inds, coefficients=None, effect="opd"):
        if not isinstance(aperture, DynamicAperture):
            raise TypeError("AberratedApertures cannot contain Static, Compound or Multi "
                            "Apertures. AberratedApertures can be placed in Compound or Multi "
                            "Apertures, which can then be promoted to Static.")
        if effect not in ("opd", "phase", "amplitude"):
            raise ValueError("effect must be 'opd', 'phase', or 'amplitude'.")
        if aperture.occulting:
            raise TypeError("AberratedApertures cannot be occulting.")
        self.aperture = aperture
        self.noll_inds = [int(j) for j in noll_inds]
        if any(j < 1 for j in self.noll_inds):
            raise ValueError("The Zernike index must be greater than 0.")
        self.effect = effect
        self.normalise = aperture.normalise
        if coefficients is None:
            coefficients = torch.zeros(len(self.noll_inds), dtype=torch.float32,
                                       device="cuda" if torch.cuda.is_available() else "cpu")
        elif not isinstance(coefficients, torch.Tensor):
            coefficients = torch.as_tensor(np.asarray(coefficients), dtype=torch.float32,
                                           device="cuda" if torch.cuda.is_available() else "cpu")
        if coefficients.shape != (len(self.noll_inds),):
            raise ValueError("coefficients must have one entry per Noll index.")
        self.coefficients = coefficients

    def _fields(self, npixels, pixel_scale):
        desc = self.aperture.desc(npixels, pixel_scale)
        trans, _ = kernels.aberrated_aperture(desc, [], None, want_opd=False)
        opd = autograd.dynamic_zernike(desc, self.noll_inds, self.coefficients)
        return trans, opd

    def eval_basis(self, npixels, pixel_scale):
        """The aberrations (OPD) at the wavefront's pixels."""
        return self._fields(npixels, pixel_scale)[1]

    def __call__(self, wavefront):
        trans, ab = self._fields(wavefront.npixels, wavefront.pixel_scale)
        wavefront *= trans
        if self.normalise:
            wavefront = wavefront.normalise()
        if self.effect == "phase":
            return wavefront.add_phase(ab)
        if self.effect == "opd":
            return wavefront.add_opd(ab)
        return wavefront * (1 + ab)

    def fuse(self, acc):
        trans, ab = self._fields(acc.n, acc.pixel_scale)
        acc.amplitude(trans)
        if self.normalise:
            acc.normalise()
        if self.effect == "opd":
            acc.add_opd(ab)
        elif self.effect == "phase":
            acc.add_phase(ab)
        else:
            acc.amplitude(1 + ab)
