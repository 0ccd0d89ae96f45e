"""ABCD-matrix propagators (dLux layers/abcd_propagators.py:1-491).

dLux composes paraxial optical elements as 2 x 2 ray-transfer (ABCD) matrices
and propagates with the linear canonical transform (LCT), or with the
angular-spectrum method (ASM) for free space. It takes that arithmetic from
the abcdLux package (``abcd``, ``lct``, ``asm``; pyproject.toml:21
"abcdLux>=0.0.2", not vendored with the reference). Here it is restated from
the published methods:

* ABCD matrices act on (position, angle) ray vectors: free space over d is
  [[1, d], [0, 1]], a thin lens of focal length f [[1, 0], [-1/f, 1]], a
  mirror of radius R [[1, 0], [-2/R, 1]], and the front-to-back focal-plane
  (Fraunhofer) system of focal length f [[0, f], [-1/f, 0]]. A sequence
  applied in order composes as M_n ... M_2 M_1.
* The LCT of an ABCD system (Collins' diffraction integral), per axis,
    u_out(x') = (i lambda B)^(-1/2) int u(x) exp(i pi / (lambda B) *
                (A x^2 - 2 x x' + D x'^2)) dx,
  sampled as a sum over the input pixels times dx. Both axes together give
  the 1 / (i lambda B) prefactor. B = 0 (an imaging condition) has no
  integral form and is rejected.
* ASM over a distance z: zero-pad, take the centred DFT, multiply by
  exp(2 pi i z sqrt(1/lambda^2 - fx^2 - fy^2)) (evanescent components decay),
  and take the inverse DFT. The pixel scale is unchanged.

Each propagation runs on the device as one of the library's plans: the LCT as
a separable two-GEMM transform with generated chirped DFT matrices
(XformPlan, the same split-BF16 tensor-core GEMMs as the MFT), and the ASM as
a DFT, a transfer-function kernel and an inverse DFT (ASMPlan). Both are
differentiable through their adjoints.
"""

from __future__ import annotations

import math

import torch

from .. import autograd, kernels
from ..base import Base
from ..coordinates import CoordSpec, PadSpec
from ..utils.array_ops import crop_to
from .optical_layers import OpticalLayer

__all__ = [
    "ABCDElement",
    "ABCDFreeSpace",
    "ABCDLens",
    "ABCDMirror",
    "ABCDConjugatePlane",
    "ABCDPropagator",
    "MFTPropagator",
    "FFTPropagator",
    "ASMPropagator",
    "Fraunhofer",
    "Fresnel",
    "abcd_free_space",
    "abcd_lens",
    "abcd_mirror",
    "abcd_fraunhofer",
    "compose_abcd",
    "abcd_effective_focal_length",
    "lct_axes",
]


# ---- ABCD matrices -----------------------------------------------------------
def _mat(a, b, c, d):
    return torch.tensor([[a, b], [c, d]], dtype=torch.float64)


def abcd_free_space(distance):
    return _mat(1.0, float(distance), 0.0, 1.0)


def abcd_lens(focal_length):
    return _mat(1.0, 0.0, -1.0 / float(focal_length), 1.0)


def abcd_mirror(radius):
    return _mat(1.0, 0.0, -2.0 / float(radius), 1.0)


def abcd_fraunhofer(focal_length):
    f = float(focal_length)
    return _mat(0.0, f, -1.0 / f, 0.0)


def compose_abcd(matrices):
    """Matrix of the elements applied in order: M_n ... M_2 M_1."""
    out = torch.eye(2, dtype=torch.float64)
    for m in matrices:
        out = torch.as_tensor(m, dtype=torch.float64) @ out
    return out


def abcd_effective_focal_length(matrix):
    """-1/C: the focal length of the equivalent thin lens (C = 0: afocal)."""
    c = float(matrix[1, 0])
    if c == 0.0:
        raise ValueError("An afocal ABCD system (C = 0) has no effective focal length.")
    return -1.0 / c


def lct_axes(matrix, wavelengths, n_in, d_in, c_in, n_out, d_out, c_out):
    """Per-wavelength LCT axes of the Collins integral on the given grids
    (x_i = c_in + (i - (n_in - 1)/2) d_in, likewise x'_j): one dict per
    wavelength, for XformPlan."""
    A, B = float(matrix[0, 0]), float(matrix[0, 1])
    D = float(matrix[1, 1])
    if B == 0.0:
        raise ValueError("The LCT of an ABCD system with B = 0 (an imaging condition) has no "
                         "integral form; it is not supported.")
    out = []
    for wl in wavelengths:
        lb = float(wl) * B
        out.append(dict(a_in=float(d_in), b_in=float(c_in) - 0.5 * (n_in - 1) * float(d_in),
                        a_out=float(d_out),
                        b_out=float(c_out) - 0.5 * (n_out - 1) * float(d_out),
                        sigma=-1.0 / lb, q_in=A / (2.0 * lb), q_out=D / (2.0 * lb),
                        phase=-0.125 if B > 0 else 0.125,
                        scale=float(d_in) / math.sqrt(abs(lb))))
    return out


# ---- elements ------------------------------------------------------------------
class ABCDElement(Base):
    """An element represented by an ABCD matrix (abcd_propagators.py:23-33)."""


class ABCDFreeSpace(ABCDElement):
    def __init__(self, distance):
        self.distance = float(distance)

    @property
    def abcd(self):
        return abcd_free_space(self.distance)


class ABCDLens(ABCDElement):
    def __init__(self, focal_length):
        self.focal_length = float(focal_length)

    @property
    def abcd(self):
        return abcd_lens(self.focal_length)


class ABCDMirror(ABCDElement):
    def __init__(self, radius):
        self.radius = float(radius)

    @property
    def abcd(self):
        return abcd_mirror(self.radius)


class ABCDConjugatePlane(ABCDElement):
    """Front-to-back focal-plane system: the pupil-focal Fourier relationship."""

    def __init__(self, focal_length):
        self.focal_length = float(focal_length)

    @property
    def abcd(self):
        return abcd_fraunhofer(self.focal_length)


def _elements(ABCDs):
    items = ABCDs.items() if isinstance(ABCDs, dict) else None
    if items is None:
        items, counts = [], {}
        for el in ABCDs:
            name = type(el).__name__
            counts[name] = counts.get(name, 0) + 1
            items.append((name if counts[name] == 1 else f"{name}_{counts[name] - 1}", el))
    out = {}
    for k, el in items:
        if not isinstance(el, ABCDElement):
            raise TypeError(f"Items must be ABCDElement instances, got {type(el)}.")
        out[k] = el
    return out


# ---- propagators -----------------------------------------------------------------
class ABCDPropagator(OpticalLayer):
    """Propagator over a composition of ABCD elements (abcd_propagators.py:191-245)."""

    def __init__(self, ABCDs, spec):
        self.ABCDs = _elements(ABCDs)
        self.spec = spec

    def __getattr__(self, key):
        d = self.__dict__
        spec = d.get("spec")
        if spec is not None and hasattr(spec, key):
            return getattr(spec, key)
        els = d.get("ABCDs", {})
        if key in els:
            return els[key]
        for el in els.values():
            if hasattr(el, key):
                return getattr(el, key)
        raise AttributeError(f"{type(self).__name__} has no attribute {key!r}.")

    @property
    def abcd(self):
        return compose_abcd([m.abcd for m in self.ABCDs.values()])


def _batch(wavefront):
    field = wavefront.phasor if wavefront.batched else wavefront.phasor[None]
    wl = wavefront.wavelengths
    if len(wl) != field.shape[0]:
        wl = wl * field.shape[0]
    return field, wl


def _unbatch(wavefront, field):
    return field if wavefront.batched else field[0]


class MFTPropagator(ABCDPropagator):
    """LCT to an explicit output grid (abcd_propagators.py:248-300): the
    Collins integral evaluated as a chirped two-GEMM transform."""

    def __call__(self, wavefront):
        spec_out = self.spec
        if spec_out.d is None or spec_out.n is None:
            raise ValueError("MFTPropagator needs an output CoordSpec with n and d.")
        c_out = 0.0 if spec_out.c is None else float(spec_out.c)
        field, wl = _batch(wavefront)
        axes = lct_axes(self.abcd, wl, wavefront.npixels, wavefront.pixel_scale,
                        wavefront.center, int(spec_out.n), float(spec_out.d), c_out)
        plan = kernels.get_xform_plan(axes, axes, wavefront.npixels, int(spec_out.n))
        out = autograd.apply_plan(plan, field.contiguous())
        return wavefront.set(phasor=_unbatch(wavefront, out), pixel_scale=float(spec_out.d),
                             center=c_out)


class FFTPropagator(ABCDPropagator):
    """LCT sampled on the FFT output grid (abcd_propagators.py:303-377).

    The output has n_padded pixels (CoordSpec n, or n * pad for a PadSpec) at
    the FFT pixel scale lambda |f| / (n_padded dx) of the system's effective
    focal length f = -1/C, centred on spec.c, then the PadSpec crop. The
    transform is the exact Collins integral on that grid (for the Fraunhofer
    system it is the focal-plane FFT), computed like MFTPropagator."""

    def __init__(self, ABCDs, spec):
        if isinstance(spec, CoordSpec) and spec.d is not None:
            raise ValueError("FFTPropagator CoordSpec can not specify d.")
        super().__init__(ABCDs=ABCDs, spec=spec)

    def __call__(self, wavefront):
        n = wavefront.npixels
        n_pad = int(self.spec.n) if isinstance(self.spec, CoordSpec) else n * self.spec.pad
        c_out = 0.0 if self.spec.c is None else float(self.spec.c)
        fl = abs(abcd_effective_focal_length(self.abcd))
        field, wl = _batch(wavefront)
        d_out = [float(w) * fl / (n_pad * wavefront.pixel_scale) for w in wl]
        A = self.abcd
        axes = []
        for w, d in zip(wl, d_out):
            axes += lct_axes(A, [w], n, wavefront.pixel_scale, wavefront.center, n_pad, d, c_out)
        plan = kernels.get_xform_plan(axes, axes, n, n_pad)
        out = autograd.apply_plan(plan, field.contiguous())
        if isinstance(self.spec, PadSpec) and self.spec.crop > 1:
            out = crop_to(out, n_pad // self.spec.crop)
        return wavefront.set(phasor=_unbatch(wavefront, out), pixel_scale=d_out[0],
                             center=c_out)


class ASMPropagator(OpticalLayer):
    """Angular-spectrum propagation over a distance (abcd_propagators.py:380-459)."""

    def __init__(self, distance, spec):
        self.distance = torch.as_tensor(float(distance), dtype=torch.float64)
        if isinstance(spec, CoordSpec) and (spec.d is not None or spec.c is not None):
            raise ValueError("ASMPropagator CoordSpec can not specify d or c.")
        self.spec = spec

    def __getattr__(self, key):
        spec = self.__dict__.get("spec")
        if spec is not None and hasattr(spec, key):
            return getattr(spec, key)
        raise AttributeError(f"{type(self).__name__} has no attribute {key!r}.")

    def __call__(self, wavefront):
        n = wavefront.npixels
        n_pad = int(self.spec.n) if isinstance(self.spec, CoordSpec) else n * self.spec.pad
        field, wl = _batch(wavefront)
        plan = kernels.get_asm_plan(wl, n, n_pad, wavefront.pixel_scale, float(self.distance))
        out = autograd.apply_plan(plan, field.contiguous())
        if isinstance(self.spec, PadSpec) and self.spec.crop > 1:
            out = crop_to(out, n_pad // self.spec.crop)
        return wavefront.set(phasor=_unbatch(wavefront, out))


class _Placeholder(ABCDPropagator):
    """A propagator without an implementation: the class itself is abstract
    (its __call__ is missing, as in dLux, so instantiating it raises
    TypeError), and a subclass that supplies __call__ still raises
    NotImplementedError from __init__."""

    def __new__(cls, *args, **kwargs):
        if "__call__" not in {k for c in cls.__mro__ if c not in _PLACEHOLDER_BASES
                              for k in vars(c)}:
            raise TypeError(f"Can't instantiate abstract class {cls.__name__} without an "
                            "implementation for abstract method '__call__'")
        return super().__new__(cls)


class Fraunhofer(_Placeholder):
    """Placeholder for a dedicated Fraunhofer propagator (abcd_propagators.py:462-475)."""

    def __init__(self):
        raise NotImplementedError("Fraunhofer propagator is not yet implemented.")


class Fresnel(_Placeholder):
    """Placeholder for a dedicated Fresnel propagator (abcd_propagators.py:478-491)."""

    def __init__(self):
        raise NotImplementedError("Fresnel propagator is not yet implemented.")


# classes whose attributes do not count as an implementation of __call__
_PLACEHOLDER_BASES = set(ABCDPropagator.__mro__) | {_Placeholder, Fraunhofer, Fresnel}
