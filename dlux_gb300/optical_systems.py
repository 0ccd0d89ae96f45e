"""Optical systems (dLux optical_systems.py:18-775).

``propagate`` keeps dLux's signature and semantics. When every layer of a
parametric layered system reduces to a wavelength-independent amplitude, OPD
and phase (the pupil-plane layers of this package), the whole polychromatic
propagation runs as one fused plan on the device: phasor build, split-BF16
(or FP32) two-step MFT and the |E|^2 wavelength sum, with a hand-written
reverse pass. Any other stack runs layer by layer on the device.
"""

from __future__ import annotations

import torch

from . import autograd, kernels
from .base import Base
from .helpers import insert_layer, list2dictionary, remove_layer
from .layers.optical_layers import NotFusable, OpticalLayer, PupilAccumulator
from .psfs import PSF
from .utils.units import arcsec2rad
from .wavefronts import Wavefront

__all__ = ["BaseOpticalSystem", "OpticalSystem", "ParametricOpticalSystem",
           "LayeredOpticalSystem", "ParametricLayeredOpticalSystem", "AngularOpticalSystem",
           "CartesianOpticalSystem"]


def _dev():
    return torch.device("cuda")


def _weights_tensor(weights, n):
    if weights is None:
        return torch.full((n,), 1.0 / n, dtype=torch.float32, device=_dev())
    w = weights if isinstance(weights, torch.Tensor) else torch.as_tensor(weights)
    w = w.to(device=_dev(), dtype=torch.float32)
    return w.reshape(-1) if w.dim() == 0 else w


class BaseOpticalSystem(Base):
    pass


class OpticalSystem(BaseOpticalSystem):
    """propagate / model shared by all systems (optical_systems.py:138-231)."""

    def propagate(self, wavelengths, offset=None, weights=None, return_wf=False,
                  return_psf=False):
        if return_wf and return_psf:
            raise ValueError("Cannot return both Wavefront and PSF objects. Choose one: "
                             "return_wf=True for Wavefront, or return_psf=True for PSF.")
        wl = torch.as_tensor(wavelengths, dtype=torch.float64).reshape(-1) \
            if not isinstance(wavelengths, torch.Tensor) else \
            wavelengths.detach().to(torch.float64).reshape(-1).cpu()
        if weights is not None:
            w_shape = tuple(torch.as_tensor(weights).shape) if not isinstance(
                weights, torch.Tensor) else tuple(weights.shape)
            if len(w_shape) == 0:
                w_shape = (1,)
            if w_shape != tuple(wl.shape):
                raise ValueError(
                    f"Wavelength and weight shape mismatch: wavelengths {tuple(wl.shape)} vs "
                    f"weights {w_shape}. Must have same length and dimensions.")
        w = _weights_tensor(weights, wl.shape[0])
        if offset is None:
            offset = torch.zeros(2, dtype=torch.float64)
        off = offset if isinstance(offset, torch.Tensor) else torch.as_tensor(offset,
                                                                              dtype=torch.float64)
        if tuple(off.shape) != (2,):
            raise ValueError(f"offset must be [x, y] array of shape (2,), got shape "
                             f"{tuple(off.shape)}. Pass offset as [on_axis_x, on_axis_y] angles "
                             "in radians.")
        wl_list = [float(v) for v in wl]
        if return_wf:
            return self._propagate_fields(wl_list, off, w)
        psf = self._propagate_psf(wl_list, off, w)
        if return_psf:
            return PSF(psf, self._psf_pixel_scale())
        return psf

    def model(self, source, return_wf=False, return_psf=False):
        return source.model(self, return_wf, return_psf)

    # hooks
    def _propagate_fields(self, wl, offset, weights):  # pragma: no cover - abstract
        raise NotImplementedError

    def _propagate_psf(self, wl, offset, weights):
        """sum_l w_l |F_l|^2 of the unweighted focal fields (weighted intensity kernel)."""
        wf = self._propagate_fields(wl, offset, None)
        f = wf.phasor if wf.phasor.dim() == 3 else wf.phasor[None]
        return autograd.psf_sum(f, weights)

    def _psf_pixel_scale(self):  # pragma: no cover - abstract
        raise NotImplementedError


class ParametricOpticalSystem(OpticalSystem):
    """PSF sampling attributes (optical_systems.py:234-292)."""

    def __init__(self, psf_npixels, psf_pixel_scale, oversample=1, **kwargs):
        self.psf_npixels = int(psf_npixels)
        self.oversample = int(oversample)
        self.psf_pixel_scale = float(psf_pixel_scale)
        super().__init__(**kwargs)

    @property
    def fov(self):
        return self.psf_npixels * self.psf_pixel_scale


class LayeredOpticalSystem(OpticalSystem):
    """Arbitrary chain of optical layers (optical_systems.py:298-507)."""

    def __init__(self, wf_npixels, diameter, layers, **kwargs):
        self.wf_npixels = int(wf_npixels)
        self.diameter = float(diameter)
        self.layers = list2dictionary(layers, True, OpticalLayer)
        super().__init__(**kwargs)

    def __getattr__(self, key):
        layers = self.__dict__.get("layers", {})
        if key in layers:
            return layers[key]
        for layer in layers.values():
            if hasattr(layer, key):
                return getattr(layer, key)
        raise AttributeError(f"{type(self).__name__} has no attribute {key!r}; layers: "
                             f"{list(layers)}")

    def initialise_wavefront(self, wavelength, offset=None):
        """1/N^2 field tilted by the source offset (optical_systems.py:363-389)."""
        if offset is None:
            offset = torch.zeros(2, dtype=torch.float64)
        wf = Wavefront(wavelength, self.wf_npixels, self.diameter)
        return wf.tilt(offset)

    def _run_layers(self, wf):
        for layer in self.layers.values():
            wf = layer(wf)
        return wf

    def _focus(self, wf):
        return wf

    def _propagate_fields(self, wl, offset, weights):
        """Focal fields of every wavelength, times sqrt(weight) when weights are given."""
        wlt = torch.tensor(wl, dtype=torch.float64)
        wf = self.initialise_wavefront(wlt, offset.detach())
        wf = self._focus(self._run_layers(wf))
        if weights is None:
            return wf
        return wf.set(phasor=wf.phasor * torch.sqrt(weights)[:, None, None])

    def propagate_mono(self, wavelength, offset=None, return_wf=False):
        """One wavelength through the layers (optical_systems.py:391-425)."""
        if return_wf:
            wf = self.initialise_wavefront(float(wavelength), offset)
            return self._focus(self._run_layers(wf))
        off = torch.zeros(2, dtype=torch.float64) if offset is None else torch.as_tensor(offset)
        return self._propagate_psf([float(wavelength)], off,
                                   torch.ones(1, dtype=torch.float32, device=_dev()))

    def debug_propagate_mono(self, wavelength, offset=None):
        outputs = {}
        wf = self.initialise_wavefront(float(wavelength), offset)
        outputs["initial_wavefront"] = wf
        for name, layer in self.layers.items():
            wf = layer(wf)
            outputs[name] = wf
        return wf, outputs

    def insert_layer(self, layer, index):
        return self.set("layers", insert_layer(self.layers, layer, index, OpticalLayer))

    def remove_layer(self, key):
        return self.set("layers", remove_layer(self.layers, key))

    def _psf_pixel_scale(self):
        return self.diameter / self.wf_npixels


class ParametricLayeredOpticalSystem(ParametricOpticalSystem, LayeredOpticalSystem):
    """Layered system ending in ``to_focus`` (optical_systems.py:510-594)."""

    def _focal_sampling(self):  # pragma: no cover - abstract
        raise NotImplementedError

    def to_focus(self, wavefront):
        npix, ps = self._focal_sampling()
        return wavefront.propagate(npix, ps)

    def _focus(self, wf):
        return self.to_focus(wf)

    def _psf_pixel_scale(self):
        return self._focal_sampling()[1]

    def debug_propagate_mono(self, wavelength, offset=None):
        wf, outputs = LayeredOpticalSystem.debug_propagate_mono(self, wavelength, offset)
        wf = self.to_focus(wf)
        outputs["final_wavefront"] = wf
        return wf, outputs

    def fused_pupil(self):
        """(amp, normalise, opd, phase, tilt, amp_scale) if every layer folds into one pupil,
        else None; amp_scale is the normalisation when it was computed alongside the OPD."""
        acc = PupilAccumulator(self.wf_npixels, pixel_scale=self.diameter / self.wf_npixels)
        try:
            for layer in self.layers.values():
                layer.fuse(acc)
        except NotFusable:
            return None
        amp, flag, opd, phase = acc.fields()
        return amp, flag, opd, phase, acc.tilt, acc.amp_scale

    def fused_plan(self, wavelengths, variant=None):
        npix, ps = self._focal_sampling()
        return kernels.get_poly_plan(wavelengths, self.wf_npixels,
                                     self.diameter / self.wf_npixels, npix, ps, None, variant)

    def _propagate_psf(self, wl, offset, weights):
        fused = self.fused_pupil()
        if fused is None:
            return OpticalSystem._propagate_psf(self, wl, offset, weights)
        amp, flag, opd, phase, tilt, amp_scale = fused
        plan = self.fused_plan(wl)
        tilt_t = offset.to(dtype=torch.float64, device=tilt.device) + tilt
        return autograd.poly_psf(plan, amp, opd, phase, weights, flag, tilt_t, amp_scale)


class AngularOpticalSystem(ParametricLayeredOpticalSystem):
    """Focal plane sampled in arcseconds (optical_systems.py:597-680)."""

    def __init__(self, wf_npixels, diameter, layers, psf_npixels, psf_pixel_scale, oversample=1):
        super().__init__(wf_npixels=wf_npixels, diameter=diameter, layers=layers,
                         psf_npixels=psf_npixels, psf_pixel_scale=psf_pixel_scale,
                         oversample=oversample)

    def _focal_sampling(self):
        return self.psf_npixels * self.oversample, arcsec2rad(self.psf_pixel_scale /
                                                              self.oversample)


class CartesianOpticalSystem(ParametricLayeredOpticalSystem):
    """Focal plane sampled in microns (optical_systems.py:683-775).

    As in dLux, to_focus scales the pixel scale by 1e-6 and propagates with
    focal_length=None (optical_systems.py:772-775).
    """

    def __init__(self, wf_npixels, diameter, layers, focal_length, psf_npixels,
                 psf_pixel_scale, oversample=1):
        self.focal_length = float(focal_length)
        super().__init__(wf_npixels=wf_npixels, diameter=diameter, layers=layers,
                         psf_npixels=psf_npixels, psf_pixel_scale=psf_pixel_scale,
                         oversample=oversample)

    def _focal_sampling(self):
        return self.psf_npixels * self.oversample, 1e-6 * self.psf_pixel_scale / self.oversample
