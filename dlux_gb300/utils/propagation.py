"""MFT and FFT propagation (dLux utils/propagation.py:8-256) on the device.

Fields are complex64 CUDA tensors of shape [N, N] or [B, N, N] (one wavelength
per batch element). The transforms run through cached plans (DFT matrices
generated on the device with FP64 phase arguments) and are differentiable: the
backward pass is the hand-written adjoint transform.
"""

from __future__ import annotations

import torch

from .. import autograd, kernels

__all__ = ["FFT", "MFT", "transfer_matrix", "calc_nfringes"]


def _wavelengths(wavelength, batch):
    wl = torch.as_tensor(wavelength, dtype=torch.float64).reshape(-1).tolist()
    if len(wl) == 1 and batch > 1:
        wl = wl * batch
    if len(wl) != batch:
        raise ValueError(f"{len(wl)} wavelengths for a batch of {batch} fields")
    return wl


def _as_field(phasor):
    t = torch.as_tensor(phasor)
    if not t.is_cuda:
        t = t.to("cuda")
    return t.to(torch.complex64)


def transfer_matrix(wavelength, npixels_in, pixel_scale_in, npixels_out, pixel_scale_out,
                    shift=0.0, focal_length=None, focal_shift=0.0, inverse=False):
    """[N_in, N_out] DFT matrix (utils/propagation.py:67-127); a batch for a wavelength array."""
    fl = None if focal_length is None else float(focal_length) + float(focal_shift)
    out = kernels.transfer_matrix(torch.as_tensor(wavelength).reshape(-1), npixels_in,
                                  pixel_scale_in, npixels_out, pixel_scale_out, shift, fl, inverse)
    return out[0] if torch.as_tensor(wavelength).dim() == 0 else out


def calc_nfringes(wavelength, npixels_in, pixel_scale_in, npixels_out, pixel_scale_out,
                  focal_length=None, focal_shift=0.0):
    """Fringes across the output plane (utils/propagation.py:130-175)."""
    out_size = npixels_out * pixel_scale_out
    if focal_length is not None:
        out_size = out_size / (focal_length + focal_shift)
    return out_size / (wavelength / (npixels_in * pixel_scale_in))


def MFT(phasor, wavelength, pixel_scale_in, npixels_out, pixel_scale_out, focal_length=None,
        shift=(0.0, 0.0), pixel=True, inverse=False):
    """Matrix Fourier transform with the dLux normalisation (utils/propagation.py:178-256)."""
    x = _as_field(phasor)
    squeeze = x.dim() == 2
    xb = x.reshape(-1, x.shape[-2], x.shape[-1])
    if xb.shape[-1] != xb.shape[-2]:
        raise ValueError("MFT expects square fields")
    shift = [float(s) for s in torch.as_tensor(shift, dtype=torch.float64).reshape(-1)]
    if len(shift) != 2:
        raise ValueError("shift must have shape (2,)")
    if not pixel:
        shift = [s / float(pixel_scale_out) for s in shift]
    wl = _wavelengths(wavelength, xb.shape[0])
    plan = kernels.get_mft_plan(wl, xb.shape[-1], float(pixel_scale_in), int(npixels_out),
                                float(pixel_scale_out), focal_length, shift, inverse)
    out = autograd.apply_plan(plan, xb)
    return out[0] if squeeze else out.reshape(*x.shape[:-2], npixels_out, npixels_out)


def FFT(phasor, wavelength, pixel_scale, focal_length=None, pad=2, inverse=False):
    """Zero-padded centred FFT (utils/propagation.py:8-64): returns (phasor, pixel_scale)."""
    x = _as_field(phasor)
    squeeze = x.dim() == 2
    xb = x.reshape(-1, x.shape[-2], x.shape[-1])
    n = xb.shape[-1]
    wl = _wavelengths(wavelength, xb.shape[0])
    fringe = torch.as_tensor(wavelength, dtype=torch.float64) / (pixel_scale * n)
    new_ps = fringe / pad
    if focal_length is not None:
        new_ps = new_ps * focal_length
    plan = kernels.get_fft_plan(wl, n, float(pixel_scale), int(pad), focal_length, inverse)
    out = autograd.apply_plan(plan, xb)
    p = kernels.fft_out_side(n, pad)
    out = out[0] if squeeze else out.reshape(*x.shape[:-2], p, p)
    return out, (float(new_ps) if new_ps.dim() == 0 else new_ps)
