"""Point sources (dLux sources.py:132-411)."""

from __future__ import annotations

import torch

from . import spectra
from .base import Base
from .psfs import PSF

__all__ = ["BaseSource", "Source", "PointSource", "PointSources", "ResolvedSource",
           "PointResolvedSource"]


def _validate_return_mode(return_wf, return_psf):
    if return_wf and return_psf:
        raise ValueError("Cannot return both Wavefront and PSF objects. Choose one: set "
                         "return_wf=True for Wavefront, or return_psf=True for PSF object.")


def _dev():
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


class BaseSource(Base):
    pass


class Source(BaseSource):
    def __init__(self, wavelengths=None, weights=None, spectrum=None):
        if spectrum is not None:
            if not isinstance(spectrum, spectra.BaseSpectrum):
                raise TypeError(f"spectrum must be a dLux BaseSpectrum instance from "
                                f"dLux.spectra, got {type(spectrum).__name__}.")
            self.spectrum = spectrum
        else:
            self.spectrum = spectra.Spectrum(wavelengths, weights)

    def __getattr__(self, key):
        spec = self.__dict__.get("spectrum")
        if spec is not None and hasattr(spec, key):
            return getattr(spec, key)
        raise AttributeError(f"{type(self).__name__} has no attribute {key!r}")

    def normalise(self):
        return self.set("spectrum", self.spectrum.normalise())


class PointSource(Source):
    """Polychromatic point source at an angular position (sources.py:132-327)."""

    def __init__(self, wavelengths=None, position=(0.0, 0.0), flux=1.0, weights=None,
                 spectrum=None):
        pos = position if isinstance(position, torch.Tensor) else torch.as_tensor(
            position, dtype=torch.float64)
        if tuple(pos.shape) != (2,):
            raise ValueError(f"position must be a 1d array of shape (2,), got shape "
                             f"{tuple(pos.shape)}. Pass position=[x, y] where x, y are on-sky "
                             "angles in radians.")
        self.position = pos
        self.flux = flux if isinstance(flux, torch.Tensor) else torch.as_tensor(
            float(flux), dtype=torch.float32, device=_dev())
        super().__init__(wavelengths=wavelengths, weights=weights, spectrum=spectrum)

    def model(self, optics, return_wf=False, return_psf=False):
        _validate_return_mode(return_wf, return_psf)
        src = self.normalise()
        weights = src.spectrum.weights * src.flux.to(src.spectrum.weights.device)
        return optics.propagate(src.spectrum.wavelengths, src.position, weights, return_wf,
                                return_psf)


class PointSources(Source):
    """Many point sources sharing one spectrum (sources.py:330-411)."""

    def __init__(self, wavelengths=None, position=((0.0, 0.0),), flux=None, weights=None,
                 spectrum=None):
        super().__init__(spectrum=spectrum, wavelengths=wavelengths, weights=weights)
        pos = position if isinstance(position, torch.Tensor) else torch.as_tensor(
            position, dtype=torch.float64)
        if pos.dim() != 2:
            raise ValueError("position must be a 2d array.")
        self.position = pos
        if flux is None:
            self.flux = torch.ones(len(pos), dtype=torch.float32, device=_dev())
        else:
            f = flux if isinstance(flux, torch.Tensor) else torch.as_tensor(
                flux, dtype=torch.float32, device=_dev())
            if f.dim() != 1:
                raise ValueError("flux must be a 1d array.")
            if len(f) != len(pos):
                raise ValueError("Length of flux must be equal to length of positions.")
            self.flux = f

    def model(self, optics, return_wf=False, return_psf=False):
        _validate_return_mode(return_wf, return_psf)
        src = self.normalise()
        w = src.spectrum.weights
        weights = w[None, :] * src.flux.to(w.device)[:, None]
        if return_wf:
            wfs = [optics.propagate(src.spectrum.wavelengths, p, wt, return_wf=True)
                   for p, wt in zip(src.position, weights)]
            return wfs[0].set(phasor=torch.stack([wf.phasor for wf in wfs]))
        psf = self._fused(optics, src, weights)
        if psf is None:
            for p, wt in zip(src.position, weights):
                one = optics.propagate(src.spectrum.wavelengths, p, wt)
                psf = one if psf is None else psf + one
        if return_psf:
            return PSF(psf, optics._psf_pixel_scale())
        return psf

    @staticmethod
    def _fused(optics, src, weights):
        """All sources in batched launches when the optics fold into one pupil."""
        from . import autograd

        if not hasattr(optics, "fused_pupil"):
            return None
        fused = optics.fused_pupil()
        if fused is None:
            return None
        amp, flag, opd, phase, tilt, _ = fused
        tilt = (float(tilt[0]), float(tilt[1]))
        wl = [float(v) for v in torch.as_tensor(src.spectrum.wavelengths,
                                               dtype=torch.float64).reshape(-1)]
        n_src = src.position.shape[0]
        npix, ps = optics._focal_sampling()
        from . import kernels
        n_in = optics.wf_npixels
        pupil_grad = any(t is not None and t.requires_grad for t in (amp, opd, phase))
        if not pupil_grad and npix <= n_in:
            # The pupil is fixed: tilt each source through its DFT matrices and
            # share one pupil field per wavelength.
            plan = kernels.get_scene_plan(wl, n_in, optics.diameter / n_in, npix, ps, None, None,
                                          max_sources=min(n_src, 32))
            return autograd.scene_psf(plan, amp, opd, phase, weights.to(torch.float32),
                                      src.position, flag, tilt)
        plan = kernels.get_poly_plan(wl, n_in, optics.diameter / n_in,
                                     npix, ps, None, None, max_objects=min(n_src, 32))
        return autograd.poly_sources(plan, amp, opd, phase, weights.to(torch.float32),
                                     src.position, flag, tilt)


_CONV_ERR = ("Wavefront information cannot be preserved through convolution. Convolution can "
             "only operate on PSFs (incoherent light). Please use return_wf=False to get the "
             "PSF array or return_psf=True to get a PSF object.")


class ResolvedSource(PointSource):
    """A point-source PSF convolved with a normalised 2-d ``distribution``
    (sources.py:414-521); the convolution runs on the device."""

    def __init__(self, wavelengths=None, position=(0.0, 0.0), flux=1.0, distribution=None,
                 weights=None, spectrum=None):
        super().__init__(wavelengths, position, flux, weights, spectrum)
        if distribution is None:
            distribution = torch.ones((3, 3), dtype=torch.float32)
        d = distribution if isinstance(distribution, torch.Tensor) else torch.as_tensor(
            distribution, dtype=torch.float32)
        if d.dim() != 2:
            raise ValueError("distribution must be a 2d array.")
        self.distribution = (d / d.sum()).to(_dev())

    def normalise(self):
        floor = torch.clamp(self.distribution, min=0.0)
        return self.set(["spectrum", "distribution"],
                        [self.spectrum.normalise(), floor / floor.sum()])

    def model(self, optics, return_wf=False, return_psf=False):
        from . import autograd
        _validate_return_mode(return_wf, return_psf)
        if return_wf:
            raise NotImplementedError(_CONV_ERR)
        src = self.normalise()
        weights = src.spectrum.weights * src.flux.to(src.spectrum.weights.device)
        psf = optics.propagate(src.spectrum.wavelengths, src.position, weights, return_psf=True)
        conv = autograd.conv2d_same(psf.data, src.distribution)
        return PSF(conv, psf.pixel_scale) if return_psf else conv


class PointResolvedSource(ResolvedSource):
    """A point source plus a resolved distribution sharing one position, with the flux
    split by ``contrast`` (sources.py:638-748, utils/source.py:8-26)."""

    def __init__(self, wavelengths=None, position=(0.0, 0.0), flux=1.0, distribution=None,
                 contrast=1.0, spectrum=None, weights=None):
        super().__init__(wavelengths, position, flux, distribution, weights, spectrum)
        self.contrast = contrast if isinstance(contrast, torch.Tensor) else torch.as_tensor(
            float(contrast), dtype=torch.float32, device=_dev())

    def model(self, optics, return_wf=False, return_psf=False):
        from . import autograd
        _validate_return_mode(return_wf, return_psf)
        if return_wf:
            raise NotImplementedError(_CONV_ERR)
        src = self.normalise()
        w = src.spectrum.weights
        c = src.contrast.to(w.device)
        flux = src.flux.to(w.device)
        # fluxes_from_contrast: 2 (contrast * mean, mean) / (1 + contrast)
        f_point = 2 * c * flux / (1 + c)
        f_resolved = 2 * flux / (1 + c)
        point = optics.propagate(src.spectrum.wavelengths, src.position, w * f_point,
                                 return_psf=True)
        resolved = optics.propagate(src.spectrum.wavelengths, src.position, w * f_resolved)
        out = point.data + autograd.conv2d_same(resolved, src.distribution)
        return PSF(out, point.pixel_scale) if return_psf else out
