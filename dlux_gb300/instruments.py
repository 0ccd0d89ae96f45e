"""Telescope (dLux instruments.py:37-171)."""

from __future__ import annotations

from .base import Base
from .detectors import BaseDetector
from .optical_systems import BaseOpticalSystem
from .psfs import PSF
from .sources import BaseSource

__all__ = ["Instrument", "Telescope"]


class Instrument(Base):
    pass


class Telescope(Instrument):
    """optics.model(source) followed by detector.model(psf) (instruments.py:140-171)."""

    def __init__(self, optics, source, detector=None):
        if not isinstance(optics, BaseOpticalSystem):
            raise TypeError(f"optics must be an OpticalSystem instance, got "
                            f"{type(optics).__name__}.")
        self.optics = optics
        if isinstance(source, tuple):
            if len(source) != 2 or not isinstance(source[1], BaseSource):
                raise TypeError("source tuple must be of the form (key: str, Source: Source).")
            source = source[1]
        if not isinstance(source, BaseSource):
            raise TypeError("source must be a Source")
        self.source = source
        if detector is not None and not isinstance(detector, BaseDetector):
            raise TypeError(f"detector must be a Detector instance, got "
                            f"{type(detector).__name__}.")
        self.detector = detector

    def __getattr__(self, key):
        for name in ("optics", "source", "detector"):
            obj = self.__dict__.get(name)
            if obj is not None and hasattr(obj, key):
                return getattr(obj, key)
        raise AttributeError(f"{type(self).__name__} has no attribute {key!r}")

    def model(self, return_psf=False):
        psfs = self.optics.model(self.source, return_psf=True)
        psf = PSF(psfs.data, psfs.pixel_scale)
        if self.detector is not None:
            return self.detector.model(psf, return_psf=return_psf)
        return psf if return_psf else psf.data
