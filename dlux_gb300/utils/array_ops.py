"""Array resizing and downsampling (dLux utils/array_ops.py:12-162)."""

from __future__ import annotations

import torch

from .. import autograd

__all__ = ["pad_to", "crop_to", "resize", "downsample"]


def _parity_msg(n_in, n, op):
    pin = "even" if n_in % 2 == 0 else "odd"
    pout = "even" if n % 2 == 0 else "odd"
    return (f"Center-preserving {op} requires parity consistency, i.e. even -> even or "
            f"odd -> odd: input array ({n_in} pixels, {pin}) cannot be {op[:-3] + 'ed'} to "
            f"{n} pixels ({pout} parity).")


def pad_to(array, npixels, fill=0.0):
    n_in = array.shape[-1]
    if n_in % 2 != npixels % 2:
        raise ValueError(_parity_msg(n_in, npixels, "padding"))
    if npixels < n_in:
        raise ValueError(f"Cannot pad to smaller size: input has {n_in} pixels, target is "
                         f"{npixels} pixels.")
    p = (npixels - n_in) // 2
    if torch.is_complex(array):
        re = torch.nn.functional.pad(array.real, (p, p, p, p), value=float(getattr(fill, "real", fill)))
        im = torch.nn.functional.pad(array.imag, (p, p, p, p), value=float(getattr(fill, "imag", 0.0)))
        return torch.complex(re, im)
    return torch.nn.functional.pad(array, (p, p, p, p), value=float(fill))


def crop_to(array, npixels):
    n_in = array.shape[-1]
    if n_in % 2 != npixels % 2:
        raise ValueError(_parity_msg(n_in, npixels, "cropping"))
    if npixels > n_in:
        raise ValueError(f"Cannot crop to larger size: input has {n_in} pixels, target is "
                         f"{npixels} pixels.")
    a, b = (n_in - npixels) // 2, (n_in + npixels) // 2
    return array[..., a:b, a:b]


def resize(array, npixels, fill=0.0):
    n_in = array.shape[-1]
    if npixels == n_in:
        return array
    if npixels < n_in:
        return crop_to(array, npixels)
    return pad_to(array, npixels, fill)


def downsample(array, n, mean=True):
    """k x k block mean or sum on the device (kernel with a hand-written reverse)."""
    if array.shape[-2] != array.shape[-1]:
        raise ValueError(f"Input array has shape {tuple(array.shape)}, which is not square")
    if array.shape[-1] % n != 0:
        raise ValueError(f"Input array has {array.shape[-1]} pixels, which is not divisible "
                         f"by {n}")
    return autograd.downsample(array.to(torch.float32), n, mean)
