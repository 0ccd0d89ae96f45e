"""Static aperture builders (dLux utils/apertures.py:153-242), host-side setup."""

from __future__ import annotations

from .coordinates import pixel_coords, to_device
from .geometry import block_reduce, circle, combine, spider
from .zernikes import zernike_basis

__all__ = ["circular_aperture"]


def circular_aperture(npixels, diameter, oversample=5, secondary_diameter=None,
                      array_diameter=None, spider_width=None, spider_angles=None,
                      zernike_nolls=None, zernike_oversize=0.01, return_support=False):
    """Transmission of a circular telescope, optionally with a masked Zernike basis."""
    if (spider_width is None) != (spider_angles is None):
        raise ValueError("`spider_width` and `spider_angles` must both be provided or both be None.")
    cd = diameter if array_diameter is None else array_diameter
    coords = pixel_coords(npixels * oversample, diameter=cd, as_numpy=True)
    layers = [circle(coords, diameter / 2)]
    if secondary_diameter is not None and secondary_diameter > 0:
        layers.append(circle(coords, secondary_diameter / 2, invert=True))
    if spider_width is not None:
        layers.append(spider(coords, spider_width, spider_angles))
    transmission = combine(layers, oversample)
    if zernike_nolls is None:
        return to_device(transmission)
    coords = pixel_coords(npixels, diameter=cd, as_numpy=True)
    basis = zernike_basis(zernike_nolls, coords, diameter * (1.0 + zernike_oversize),
                          as_numpy=True)
    support = block_reduce(layers[0], oversample) > 0
    basis = basis * support[None]
    if return_support:
        return to_device(transmission), to_device(basis), to_device(support)
    return to_device(transmission), to_device(basis)
