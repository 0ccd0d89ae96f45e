"""Wavefront state and propagation (dLux wavefronts.py:17-922) on the device.

A ``Wavefront`` holds a complex64 CUDA field of shape [N, N], or [B, N, N]
for a batch of wavelengths (the layout dLux produces by vmapping over
wavelength), together with its wavelength(s), pixel scale and centre. Every
update returns a new object, as in dLux.
"""

from __future__ import annotations

import math

import torch

from . import autograd, kernels
from .base import Base
from .coordinates import CoordSpec
from .psfs import PSF
from .utils import array_ops
from .utils.fourier import fft_spec
from .utils.units import unit_factor_to_rad

__all__ = ["Wavefront"]


def _wl_list(wavelength):
    return [float(w) for w in torch.as_tensor(wavelength, dtype=torch.float64).reshape(-1)]


class Wavefront(Base):
    """Complex field of a square grid at one or several wavelengths."""

    def __init__(self, wavelength, npixels, diameter=None, pixel_scale=None, center=None):
        if diameter is None and pixel_scale is None:
            raise ValueError("Provide one: diameter or pixel_scale.")
        if diameter is not None and pixel_scale is not None:
            raise ValueError(
                "Cannot specify both 'diameter' and 'pixel_scale' - they are interdependent "
                "(diameter = pixel_scale × npixels). Choose one: use 'diameter' for wavefront "
                "diameter, or 'pixel_scale' for wavefront sampling.")
        npixels = int(npixels)
        self.wavelength = wavelength if isinstance(wavelength, torch.Tensor) and \
            wavelength.dim() else float(wavelength)
        self.pixel_scale = float(diameter) / npixels if diameter is not None else float(pixel_scale)
        wl = _wl_list(wavelength)
        # 1/N^2 amplitude, zero phase (wavefronts.py:111-113), built on the device
        field = kernels.phasor(wl, npixels, self.pixel_scale, const_scale=1.0 / npixels ** 2)
        self.phasor = field if isinstance(self.wavelength, torch.Tensor) else field[0]
        if center is not None:
            c = torch.as_tensor(center, dtype=torch.float64).reshape(-1)
            if c.shape != (1,):
                raise ValueError("center must have shape (1,).")
            self.center = float(c[0])
        else:
            self.center = 0.0

    @classmethod
    def from_phasor(cls, phasor, wavelength, pixel_scale=None, diameter=None, center=None):
        phasor = torch.as_tensor(phasor, dtype=torch.complex64, device="cuda")
        wf = cls(wavelength, phasor.shape[-1], diameter=diameter, pixel_scale=pixel_scale,
                 center=center)
        return wf.set(phasor=phasor)

    # ---- derived quantities ----
    @property
    def npixels(self):
        return self.phasor.shape[-1]

    @property
    def diameter(self):
        return self.npixels * self.pixel_scale

    @property
    def wavelengths(self):
        return _wl_list(self.wavelength)

    @property
    def batched(self):
        return self.phasor.dim() == 3

    @property
    def real(self):
        return self.phasor.real

    @property
    def imaginary(self):
        return self.phasor.imag

    @property
    def amplitude(self):
        return self.phasor.abs()

    @property
    def phase(self):
        return self.phasor.angle()

    @property
    def complex(self):
        return torch.stack([self.phasor.real, self.phasor.imag], 0)

    @property
    def polar(self):
        return torch.stack([self.amplitude, self.phase], 0)

    @property
    def psf(self):
        return self.phasor.real ** 2 + self.phasor.imag ** 2

    def to_psf(self):
        return PSF(self.psf, self.pixel_scale)

    @property
    def wavenumber(self):
        if isinstance(self.wavelength, torch.Tensor):
            return 2 * math.pi / self.wavelength
        return 2 * math.pi / self.wavelength

    @property
    def ndim(self):
        return 1 if self.batched else 0

    @property
    def power(self):
        return (self.phasor.real ** 2 + self.phasor.imag ** 2).sum((-2, -1))

    @property
    def spec(self):
        return CoordSpec(self.npixels, self.pixel_scale, self.center)

    @property
    def xs(self):
        return self.spec.xs

    def coordinates(self, scale=1.0, polar=False):
        xs = (self.xs * scale).to(torch.float32).to(self.phasor.device)
        yy, xx = torch.meshgrid(xs, xs, indexing="ij")
        coords = torch.stack([xx, yy])
        if polar:
            return torch.stack([torch.hypot(coords[0], coords[1]),
                                torch.atan2(coords[1], coords[0])])
        return coords

    # ---- elementwise updates (phasor kernel) ----
    def _mul_phasor(self, amp=None, opd=None, phase=None):
        field = self.phasor if self.batched else self.phasor[None]
        wl = self.wavelengths
        if len(wl) == 1 and field.shape[0] > 1:
            wl = wl * field.shape[0]
        out = autograd.PhasorMul.apply(tuple(wl), self.pixel_scale, field.contiguous(),
                                       _f32(amp, field.device), _f32(opd, field.device),
                                       _f32(phase, field.device))
        return self.set(phasor=out if self.batched else out[0])

    def add_phase(self, phase):
        """phasor *= exp(1j * phase) (wavefronts.py:332-349)."""
        if phase is None:
            return self
        return self._mul_phasor(phase=phase)

    def add_opd(self, opd):
        """phasor *= exp(1j * k * opd) (wavefronts.py:351-368)."""
        if opd is None:
            return self
        return self._mul_phasor(opd=opd)

    def tilt(self, angles, unit="rad"):
        """Tilt by (x, y) angles (wavefronts.py:370-395); differentiable in the angles."""
        a = torch.as_tensor(angles, dtype=torch.float64)
        if a.shape != (2,):
            raise ValueError("angles must be a 1d array of shape (2,).")
        f = unit_factor_to_rad(unit)
        differentiable = isinstance(angles, torch.Tensor) and angles.requires_grad
        if not differentiable and float(a[0]) == 0.0 and float(a[1]) == 0.0:
            # exp(i 0) = 1 exactly: the field is unchanged (and no coordinate
            # grid is built, so the step stays capturable as a CUDA graph)
            return self
        coords = self.coordinates()
        if differentiable:
            at = (angles.to(torch.float64) * f).to(device=coords.device, dtype=torch.float32)
            opd = at[0] * coords[0] + at[1] * coords[1]
        else:
            opd = (float(a[0]) * f) * coords[0] + (float(a[1]) * f) * coords[1]
        return self.add_opd(opd)

    def normalise(self, mode="power", value=1.0):
        """Scale each wavelength's field to unit power or unit peak (wavefronts.py:397-424):
        the normalisation kernel and its hand-written reverse pass."""
        if mode not in ("power", "peak"):
            raise ValueError("mode must be 'power' or 'peak'")
        return self.set(phasor=autograd.normalise(self.phasor, mode, value))

    def flip(self, axis):
        return self.set(phasor=torch.flip(self.phasor, dims=(axis,) if isinstance(axis, int)
                                          else tuple(axis)))

    def resize(self, npixels):
        return self.set(phasor=array_ops.resize(self.phasor, npixels, 0j))

    def set_spec(self, spec):
        return self.set(pixel_scale=self.pixel_scale if spec.d is None else float(spec.d),
                        center=self.center if spec.c is None else float(spec.c))

    # ---- propagation ----
    def propagate(self, npixels, pixel_scale, focal_length=None, inverse=False):
        """MFT propagation (wavefronts.py:729-772)."""
        from .utils.propagation import MFT

        out = MFT(self.phasor, self.wavelengths if self.batched else self.wavelength,
                  self.pixel_scale, int(npixels), float(pixel_scale), focal_length,
                  inverse=inverse)
        return self.set(phasor=out, pixel_scale=float(pixel_scale))

    def propagate_MFT(self, spec_out, focal_length=None, inverse=None):
        """MFT propagation with a CoordSpec (wavefronts.py:774-805)."""
        return self.propagate(spec_out.n, spec_out.d, focal_length, bool(inverse))

    def propagate_FFT(self, pad=2, focal_length=None, spec_out=None, inverse=False):
        """FFT propagation with optional centring ramps (wavefronts.py:654-727)."""
        n_out = self.npixels * pad
        wl = self.wavelengths
        d_fft, c_fft = fft_spec(n_out, self.pixel_scale, wl[0], focal_length)
        if spec_out is not None:
            if kernels.fft_out_side(self.npixels, pad) != n_out:
                # dLux's ramp of n_out pixels does not broadcast against its FFT output
                raise ValueError(f"the FFT of {self.npixels} pixels padded by {pad} has "
                                 f"{kernels.fft_out_side(self.npixels, pad)} pixels, not "
                                 f"{n_out}: output ramps need npixels * (pad - 1) even")
            if spec_out.d is not None:
                raise ValueError("Output spec cannot specify d; FFT output d is fixed.")
            if spec_out.n is not None:
                raise ValueError("Output spec cannot specify n; FFT output n is determined by "
                                 "the pad parameter.")
            ramps = (self.center, spec_out.c)
            c_out = spec_out.c
        else:
            ramps = None
            c_out = c_fft
        field = self.phasor if self.batched else self.phasor[None]
        plan = kernels.get_fft_plan(wl if len(wl) == field.shape[0] else wl * field.shape[0],
                                    self.npixels, self.pixel_scale, int(pad), focal_length,
                                    inverse, ramps)
        out = autograd.apply_plan(plan, field.contiguous())
        ps = [fft_spec(n_out, self.pixel_scale, w, focal_length)[0] for w in wl]
        pixel_scale = ps[0] if len(ps) == 1 else ps[0]
        return self.set(phasor=out if self.batched else out[0], pixel_scale=pixel_scale,
                        center=c_out)

    # ---- arithmetic ----
    def _op(self, other, op):
        if other is None:
            return self
        if isinstance(other, Wavefront):
            other = other.phasor
        if not isinstance(other, (torch.Tensor, float, int, complex)):
            raise TypeError(f"Unsupported type for {op}: {type(other)}. Must be an array, "
                            "Wavefront, or None.")
        if op == "multiply" and isinstance(other, torch.Tensor) and not torch.is_complex(other) \
                and other.shape == self.phasor.shape[-2:]:
            return self._mul_phasor(amp=other)
        if op == "add":
            return self.set(phasor=self.phasor + other)
        if op == "subtract":
            return self.set(phasor=self.phasor - other)
        if op == "multiply":
            return self.set(phasor=self.phasor * other)
        if op == "divide":
            return self.set(phasor=self.phasor / other)
        raise ValueError(f"Unsupported operation '{op}'.")

    def __add__(self, o): return self._op(o, "add")
    def __sub__(self, o): return self._op(o, "subtract")
    def __mul__(self, o): return self._op(o, "multiply")
    def __truediv__(self, o): return self._op(o, "divide")
    __iadd__ = __add__
    __isub__ = __sub__
    __imul__ = __mul__
    __itruediv__ = __truediv__


def _f32(x, device):
    if x is None:
        return None
    t = torch.as_tensor(x, device=device)
    return t.to(torch.float32).contiguous()
