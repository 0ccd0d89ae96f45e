"""Dynamic apertures evaluated on the device (layers/apertures.py of dLux).

``CircularAperture`` is a soft-edged disk under an optional ``CoordTransform``
(layers/apertures.py:240-312, utils/geometry.py:49-91 and :229-255).
``AberratedAperture`` adds Zernike aberrations defined on that aperture
(layers/apertures.py:643-800; polynomials.py:20-51). Both are computed per
pixel by ``dlx_aberrated_aperture``, with no stored basis. The OPD is
differentiable with respect to the coefficients; the aperture geometry is a
constant here.

Only circular apertures are implemented. dLux's polygonal apertures use
polygon-orthogonalised Zernikes (``polike``).
"""

from __future__ import annotations

import numpy as np
import torch

from .. import autograd, kernels
from ..base import Base
from .optical_layers import OpticalLayer

__all__ = ["CoordTransform", "CircularAperture", "AberratedAperture"]


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


class CircularAperture(OpticalLayer):
    """Soft-edged circle of ``radius`` (m) (layers/apertures.py:240-312)."""

    def __init__(self, radius, transformation=None, occulting=False, softening=1.0,
                 normalise=False):
        if transformation is not None and not isinstance(transformation, CoordTransform):
            raise TypeError("transformation must be a BaseCoordTransform instance, got "
                            f"{type(transformation).__name__}.")
        if float(softening) <= 0:
            raise ValueError("softening must be greater than 0.")
        self.radius = float(radius)
        self.transformation = transformation
        self.occulting = bool(occulting)
        self.softness = float(softening)
        self.normalise = bool(normalise)

    @property
    def extent(self):
        return self.radius

    @property
    def nsides(self):
        return 0

    def desc(self, npixels, pixel_scale):
        t = self.transformation
        return kernels.aperture_desc(npixels, pixel_scale, self.radius, self.softness,
                                     self.occulting,
                                     None if t is None else t.translation,
                                     None if t is None else t.rotation,
                                     None if t is None else t.compression,
                                     None if t is None else t.shear)

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


class AberratedAperture(OpticalLayer):
    """Zernike aberrations on a dynamic aperture (layers/apertures.py:643-800)."""

    def __init__(self, aperture, noll_inds, coefficients=None, effect="opd"):
        if not isinstance(aperture, CircularAperture):
            raise TypeError("AberratedApertures cannot contain Static, Compound or Multi "
                            "Apertures (only circular dynamic apertures are supported here).")
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
