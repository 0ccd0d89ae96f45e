"""Layered detector (dLux detectors.py:13-173)."""

from __future__ import annotations

from . import autograd
from .base import Base
from .helpers import insert_layer, list2dictionary, remove_layer
from .layers.detector_layers import ApplyPixelResponse, DetectorLayer, Downsample

__all__ = ["BaseDetector", "LayeredDetector"]


class BaseDetector(Base):
    def model(self, psf, return_psf=False):
        return self(psf, return_psf)


class LayeredDetector(BaseDetector):
    """Applies detector layers in order (detectors.py:103-128).

    A Downsample layer directly followed by an ApplyPixelResponse layer runs as
    one fused device kernel (block sum times flat field).
    """

    def __init__(self, layers):
        self.layers = list2dictionary(layers, True, DetectorLayer)

    def __getattr__(self, key):
        layers = self.__dict__.get("layers", {})
        if key in layers:
            return layers[key]
        for layer in layers.values():
            if hasattr(layer, key):
                return getattr(layer, key)
        raise AttributeError(f"{type(self).__name__} has no attribute {key!r}; layers: "
                             f"{list(layers)}")

    def __call__(self, psf, return_psf=False):
        layers = list(self.layers.values())
        i = 0
        while i < len(layers):
            layer = layers[i]
            nxt = layers[i + 1] if i + 1 < len(layers) else None
            if isinstance(layer, Downsample) and isinstance(nxt, ApplyPixelResponse):
                k = layer.kernel_size
                psf = psf.set(data=autograd.downsample(psf.data, k, False, nxt.pixel_response),
                              pixel_scale=psf.pixel_scale * k)
                i += 2
                continue
            psf = layer(psf)
            i += 1
        return psf if return_psf else psf.data

    def insert_layer(self, layer, index):
        return self.set("layers", insert_layer(self.layers, layer, index, DetectorLayer))

    def remove_layer(self, key):
        return self.set("layers", remove_layer(self.layers, key))
