"""Pixel-coordinate helpers (dLux utils/coordinates.py:166-341), host-side setup.

These build wavelength-independent grids once per configuration; they run in
float64 NumPy and return float32 tensors on the CUDA device when one is present.
"""

from __future__ import annotations

import numpy as np
import torch

__all__ = ["nd_coords", "pixel_coords", "cart2polar", "polar2cart", "to_device"]


def to_device(a, dtype=torch.float32):
    """Tensor on the current CUDA device (host tensor only when no device exists)."""
    dev = torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=dtype)
    return torch.as_tensor(np.asarray(a), dtype=dtype, device=dev)


def _linspace(n, scale, offset):
    # utils/coordinates.py:325-330 (pixel_fn)
    return np.linspace(-(n - 1) / 2 * scale - offset, (n - 1) / 2 * scale - offset, n)


def nd_coords(npixels, pixel_scales=1.0, offsets=0.0, indexing="xy", as_numpy=False):
    """Centred pixel coordinates, meshgridded for more than one dimension."""
    if indexing not in ("xy", "ij"):
        raise ValueError("indexing must be either 'xy' or 'ij'.")
    npix = (npixels,) if np.isscalar(npixels) else tuple(npixels)
    ps = np.atleast_1d(np.asarray(pixel_scales, float))
    off = np.atleast_1d(np.asarray(offsets, float))
    ndim = max(len(npix), len(ps), len(off))
    if len(npix) != ndim:
        npix = npix * ndim
    ps = np.broadcast_to(ps, (ndim,))
    off = np.broadcast_to(off, (ndim,))
    lins = [_linspace(int(n), float(s), float(o)) for n, s, o in zip(npix, ps, off)]
    out = np.squeeze(np.array(np.meshgrid(*lins, indexing=indexing)))
    return out if as_numpy else to_device(out)


def pixel_coords(npixels, diameter=None, radius=None, pixel_scale=None, polar=False,
                 fft_style=False, as_numpy=False):
    """(x, y) pixel-centre grid of a square array (utils/coordinates.py:208-266)."""
    supplied = sum(v is not None for v in (diameter, radius, pixel_scale))
    if supplied != 1:
        raise ValueError("Exactly one of diameter, radius, or pixel_scale must be provided.")
    if diameter is not None:
        pixscale = diameter / npixels
    elif radius is not None:
        pixscale = 2 * radius / npixels
    else:
        pixscale = pixel_scale
    offsets = (0.0, 0.0)
    if fft_style and npixels % 2 == 0:
        offsets = (pixscale / 2.0, pixscale / 2.0)
    coords = nd_coords((npixels,) * 2, (pixscale,) * 2, offsets, "xy", as_numpy=True)
    if polar:
        coords = cart2polar(coords)
    return coords if as_numpy else to_device(coords)


def cart2polar(coords):
    x, y = coords[0], coords[1]
    if isinstance(coords, torch.Tensor):
        return torch.stack([torch.hypot(x, y), torch.atan2(y, x)])
    return np.array([np.hypot(x, y), np.arctan2(y, x)])


def polar2cart(coords):
    r, phi = coords[0], coords[1]
    if isinstance(coords, torch.Tensor):
        return torch.stack([r * torch.cos(phi), r * torch.sin(phi)])
    return np.array([r * np.cos(phi), r * np.sin(phi)])
