"""Tensor-level wrappers of the C ABI: one function or plan class per entry point.

All inputs and outputs are CUDA tensors (float32, complex64). Work is enqueued
on torch's current stream. Shapes follow dLux: square fields, axis 0 = y.
"""

from __future__ import annotations

import collections
import ctypes
import math
import threading

import torch

from . import _lib
from ._lib import call, ptr, stream_ptr

_variant_lock = threading.Lock()
_default_variant = None


def tensor_core_available() -> bool:
    """True when the split-BF16 tcgen05 form can run on the current device."""
    if not torch.cuda.is_available():
        return False
    major, minor = torch.cuda.get_device_capability()
    return (major, minor) == (10, 3)


def set_variant(name: str | None) -> None:
    """Select the MFT arithmetic form: "split_bf16", "fp32", or None (automatic)."""
    global _default_variant
    if name not in (None, "split_bf16", "fp32"):
        raise ValueError("variant must be 'split_bf16', 'fp32' or None")
    with _variant_lock:
        _default_variant = name


def get_variant() -> str | None:
    return _default_variant


def fft_out_side(n_in: int, pad: int) -> int:
    """Side of dLux's padded FFT output: n_in zero-padded by (n_in (pad - 1)) // 2 on
    each side (utils/propagation.py:52-53)."""
    return int(n_in) + 2 * ((int(n_in) * (int(pad) - 1)) // 2)


def resolve_variant(n_in: int, n_out: int, variant: str | None = None) -> int:
    """Integer variant for a transform of the given sides.

    Automatic choice: the split-BF16 tensor-core form on sm_103a (split operands
    pad their rows to a multiple of 8 elements, so every side runs on the tensor
    cores), the FP32 form otherwise.
    """
    v = variant if variant is not None else _default_variant
    if isinstance(v, int) and v in (_lib.VARIANT_FP32, _lib.VARIANT_SPLIT_BF16):
        return v
    if v == "fp32":
        return _lib.VARIANT_FP32
    if v == "split_bf16":
        return _lib.VARIANT_SPLIT_BF16
    if tensor_core_available():
        return _lib.VARIANT_SPLIT_BF16
    return _lib.VARIANT_FP32


def _stream():
    return stream_ptr()


def _contig(t):
    return None if t is None else t.contiguous()


def _f32(x, device=None):
    dev = device or _lib.require_cuda()
    return torch.as_tensor(x, dtype=torch.float32, device=dev).contiguous()


def _c64(x, device=None):
    dev = device or _lib.require_cuda()
    return torch.as_tensor(x, dtype=torch.complex64, device=dev).contiguous()


# ---------------------------------------------------------------------------
# a1: transfer matrix
# ---------------------------------------------------------------------------
def transfer_matrix(wavelengths, npixels_in, pixel_scale_in, npixels_out, pixel_scale_out,
                    shift=0.0, focal_length=None, inverse=False, transpose=False):
    """[B, N_in, N_out] complex64 DFT matrices (dLux utils/propagation.py:67-127)."""
    dev = _lib.require_cuda()
    wl = [float(w) for w in torch.as_tensor(wavelengths, dtype=torch.float64).reshape(-1)]
    shape = (len(wl), npixels_out, npixels_in) if transpose else (len(wl), npixels_in, npixels_out)
    out = torch.empty(shape, dtype=torch.complex64, device=dev)
    call("dlx_transfer_matrix", _lib.dbl_array(wl), len(wl), int(npixels_in),
         float(pixel_scale_in), int(npixels_out), float(pixel_scale_out), float(shift),
         float(focal_length) if focal_length is not None else 0.0, int(bool(inverse)),
         int(bool(transpose)), ptr(out), _stream())
    return out


# ---------------------------------------------------------------------------
# Plan caches
# ---------------------------------------------------------------------------
class _PlanCache:
    """Small LRU of device plans keyed by their full description."""

    def __init__(self, capacity: int):
        self.capacity = capacity
        self._d = collections.OrderedDict()
        self._lock = threading.Lock()

    def get(self, key, factory):
        with self._lock:
            if key in self._d:
                self._d.move_to_end(key)
                return self._d[key]
        plan = factory()
        with self._lock:
            self._d[key] = plan
            self._d.move_to_end(key)
            while len(self._d) > self.capacity:
                _, old = self._d.popitem(last=False)
                old.close()
        return plan

    def clear(self):
        with self._lock:
            items = list(self._d.values())
            self._d.clear()
        for p in items:
            p.close()


class _Plan:
    _destroy = None

    def __init__(self):
        self.handle = ctypes.c_void_p()

    def close(self):
        if self.handle and self.handle.value:
            try:
                torch.cuda.current_stream().synchronize()
            except Exception:  # pragma: no cover - interpreter shutdown
                pass
            getattr(_lib.load(), self._destroy)(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass


class MFTPlan(_Plan):
    """Batched MFT with cached DFT matrices (dLux utils/propagation.py:178-256)."""

    _destroy = "dlx_mft_plan_destroy"

    def __init__(self, wavelengths, n_in, pixel_scale_in, n_out, pixel_scale_out,
                 focal_length=None, shift=(0.0, 0.0), inverse=False, variant=None):
        super().__init__()
        _lib.require_cuda()
        self.wavelengths = tuple(float(w) for w in wavelengths)
        self.n_in, self.n_out = int(n_in), int(n_out)
        self.variant = resolve_variant(self.n_in, self.n_out, variant)
        d = _lib.MftDesc(len(self.wavelengths), self.n_in, self.n_out, float(pixel_scale_in),
                         float(pixel_scale_out),
                         float(focal_length) if focal_length is not None else 0.0,
                         float(shift[0]), float(shift[1]), int(bool(inverse)), self.variant)
        call("dlx_mft_plan_create", ctypes.byref(d), _lib.dbl_array(self.wavelengths),
             ctypes.byref(self.handle))

    def forward(self, phasor):
        b = len(self.wavelengths)
        x = phasor.reshape(b, self.n_in, self.n_in).contiguous()
        out = torch.empty((b, self.n_out, self.n_out), dtype=torch.complex64, device=x.device)
        call("dlx_mft_forward", self.handle, ptr(x), ptr(out), _stream())
        return out

    def adjoint(self, gout):
        b = len(self.wavelengths)
        g = gout.reshape(b, self.n_out, self.n_out).contiguous()
        out = torch.empty((b, self.n_in, self.n_in), dtype=torch.complex64, device=g.device)
        call("dlx_mft_adjoint", self.handle, ptr(g), ptr(out), _stream())
        return out


class XformPlan(_Plan):
    """Separable transform out = A_y in A_x^T with generated matrices whose axes
    carry affine and quadratic phase terms (the linear canonical transform of
    an ABCD system): the device side of dLux's MFTPropagator/FFTPropagator
    (layers/abcd_propagators.py:245-370).

    ``axes_x`` / ``axes_y``: one dict per batch element with keys a_in, b_in,
    a_out, b_out, sigma, q_in, q_out, phase, scale (see dlx_xform_axis)."""

    _destroy = "dlx_xform_plan_destroy"

    def __init__(self, axes_x, axes_y, n_in, n_out, variant=None):
        super().__init__()
        _lib.require_cuda()
        self.batch = len(axes_x)
        if len(axes_y) != self.batch or self.batch == 0:
            raise ValueError("axes_x and axes_y need the same, non-zero length")
        self.n_in, self.n_out = int(n_in), int(n_out)
        self.variant = resolve_variant(self.n_in, self.n_out, variant)
        arr = _lib.XformAxis * self.batch
        ax = arr(*[_lib.XformAxis(**{k: float(v) for k, v in a.items()}) for a in axes_x])
        ay = arr(*[_lib.XformAxis(**{k: float(v) for k, v in a.items()}) for a in axes_y])
        d = _lib.XformDesc(self.batch, self.n_in, self.n_out, self.variant)
        call("dlx_xform_plan_create", ctypes.byref(d), ctypes.cast(ax, ctypes.c_void_p),
             ctypes.cast(ay, ctypes.c_void_p), ctypes.byref(self.handle))

    def forward(self, phasor):
        x = phasor.reshape(self.batch, self.n_in, self.n_in).contiguous()
        out = torch.empty((self.batch, self.n_out, self.n_out), dtype=torch.complex64,
                          device=x.device)
        call("dlx_xform_forward", self.handle, ptr(x), ptr(out), _stream())
        return out

    def adjoint(self, gout):
        g = gout.reshape(self.batch, self.n_out, self.n_out).contiguous()
        out = torch.empty((self.batch, self.n_in, self.n_in), dtype=torch.complex64,
                          device=g.device)
        call("dlx_xform_adjoint", self.handle, ptr(g), ptr(out), _stream())
        return out


class ASMPlan(_Plan):
    """Angular-spectrum propagation over ``distance`` of fields padded from n_in
    to n_pad pixels (the ASMPropagator of layers/abcd_propagators.py:380-459)."""

    _destroy = "dlx_asm_plan_destroy"

    def __init__(self, wavelengths, n_in, n_pad, pixel_scale, distance, variant=None):
        super().__init__()
        _lib.require_cuda()
        self.wavelengths = tuple(float(w) for w in wavelengths)
        self.n_in, self.n_pad = int(n_in), int(n_pad)
        self.variant = resolve_variant(self.n_in, self.n_pad, variant)
        d = _lib.AsmDesc(len(self.wavelengths), self.n_in, self.n_pad, float(pixel_scale),
                         float(distance), self.variant)
        call("dlx_asm_plan_create", ctypes.byref(d), _lib.dbl_array(self.wavelengths),
             ctypes.byref(self.handle))

    def forward(self, phasor):
        b = len(self.wavelengths)
        x = phasor.reshape(b, self.n_in, self.n_in).contiguous()
        out = torch.empty((b, self.n_pad, self.n_pad), dtype=torch.complex64, device=x.device)
        call("dlx_asm_forward", self.handle, ptr(x), ptr(out), _stream())
        return out

    def adjoint(self, gout):
        b = len(self.wavelengths)
        g = gout.reshape(b, self.n_pad, self.n_pad).contiguous()
        out = torch.empty((b, self.n_in, self.n_in), dtype=torch.complex64, device=g.device)
        call("dlx_asm_adjoint", self.handle, ptr(g), ptr(out), _stream())
        return out


def get_xform_plan(axes_x, axes_y, n_in, n_out, variant=None):
    key = ("xform", tuple(tuple(sorted(a.items())) for a in axes_x),
           tuple(tuple(sorted(a.items())) for a in axes_y), int(n_in), int(n_out),
           resolve_variant(int(n_in), int(n_out), variant))
    return xform_plans.get(key, lambda: XformPlan(axes_x, axes_y, n_in, n_out, variant))


def get_asm_plan(wavelengths, n_in, n_pad, pixel_scale, distance, variant=None):
    key = ("asm", tuple(float(w) for w in wavelengths), int(n_in), int(n_pad),
           float(pixel_scale), float(distance), resolve_variant(int(n_in), int(n_pad), variant))
    return xform_plans.get(key, lambda: ASMPlan(wavelengths, n_in, n_pad, pixel_scale,
                                                distance, variant))


# pad * N from which the padded FFT runs as radix-2 line FFTs instead of the
# DFT-GEMM pair, whose cost grows as P^2 N. Measured forward + adjoint of 16
# wavelengths: P = 1024 0.54 ms (split-BF16 GEMM) vs 0.70 ms (radix); P = 2048
# 3.08 vs 2.89 ms; P = 4096 24.3 vs 15.3 ms. Without tensor cores (FP32 GEMM
# form) the radix form is faster at every measured size.
RADIX_FFT_MIN = 2048


def resolve_fft_variant(n_in, pad, variant=None):
    """Integer form of an FFT plan: "radix" (power-of-two pad * N <= 8192), or the
    MFT forms. Automatic: radix from RADIX_FFT_MIN on, otherwise as resolve_variant."""
    p = fft_out_side(n_in, pad)
    pow2 = p == int(n_in) * int(pad) and p & (p - 1) == 0 and p <= 8192
    if variant == "radix" or variant == _lib.VARIANT_RADIX:
        if not pow2:
            raise ValueError("the radix FFT form needs pad * npixels to be a power of two <= 8192")
        return _lib.VARIANT_RADIX
    if variant is None and _default_variant is None and pow2:
        if p >= RADIX_FFT_MIN or (p >= 512 and not tensor_core_available()):
            return _lib.VARIANT_RADIX
    return resolve_variant(n_in, p, variant)


class FFTPlan(_Plan):
    """Padded centred FFT (dLux utils/propagation.py:8-64): a DFT-GEMM pair, or
    radix-2 line FFTs for large power-of-two pad * N."""

    _destroy = "dlx_fft_plan_destroy"

    def __init__(self, wavelengths, n_in, pixel_scale_in, pad=2, focal_length=None,
                 inverse=False, ramps=None, variant=None):
        super().__init__()
        _lib.require_cuda()
        self.wavelengths = tuple(float(w) for w in wavelengths)
        self.n_in, self.pad = int(n_in), int(pad)
        self.n_out = fft_out_side(self.n_in, self.pad)
        self.variant = resolve_fft_variant(self.n_in, self.pad, variant)
        apply, c_in, c_out = (0, 0.0, 0.0) if ramps is None else (1, float(ramps[0]),
                                                                 float(ramps[1]))
        d = _lib.FftDesc(len(self.wavelengths), self.n_in, self.pad, float(pixel_scale_in),
                         float(focal_length) if focal_length is not None else 0.0,
                         int(bool(inverse)), apply, c_in, c_out, self.variant)
        call("dlx_fft_plan_create", ctypes.byref(d), _lib.dbl_array(self.wavelengths),
             ctypes.byref(self.handle))

    def forward(self, phasor):
        b = len(self.wavelengths)
        x = phasor.reshape(b, self.n_in, self.n_in).contiguous()
        out = torch.empty((b, self.n_out, self.n_out), dtype=torch.complex64, device=x.device)
        call("dlx_fft_forward", self.handle, ptr(x), ptr(out), _stream())
        return out

    def adjoint(self, gout):
        b = len(self.wavelengths)
        g = gout.reshape(b, self.n_out, self.n_out).contiguous()
        out = torch.empty((b, self.n_in, self.n_in), dtype=torch.complex64, device=g.device)
        call("dlx_fft_adjoint", self.handle, ptr(g), ptr(out), _stream())
        return out


class PolyPlan(_Plan):
    """Fused polychromatic PSF and its gradient (OpticalSystem.propagate)."""

    _destroy = "dlx_poly_plan_destroy"

    def __init__(self, wavelengths, n_in, pixel_scale_in, n_out, pixel_scale_out,
                 focal_length=None, variant=None, max_objects=1, operand_mode=0,
                 own_workspace=True, gemm_pair=None, split_k=True):
        """gemm_pair: None follows the process-wide paired-GEMM switch, False never
        pairs, True pairs where the shape allows; split_k False keeps every GEMM
        whole (see dlx_poly_plan_set_gemm_form)."""
        super().__init__()
        _lib.require_cuda()
        self.wavelengths = tuple(float(w) for w in wavelengths)
        self.n_in, self.n_out = int(n_in), int(n_out)
        self.pixel_scale_in = float(pixel_scale_in)
        self.max_objects = int(max_objects)
        self.variant = resolve_variant(self.n_in, self.n_out, variant)
        self.operand_mode = int(operand_mode) if self.variant == _lib.VARIANT_SPLIT_BF16 else 0
        self.desc = _lib.PolyDesc(len(self.wavelengths), self.n_in, self.n_out,
                                  float(pixel_scale_in), float(pixel_scale_out),
                                  float(focal_length) if focal_length is not None else 0.0,
                                  self.variant, self.operand_mode)
        fn = "dlx_poly_plan_create_batched" if own_workspace else "dlx_poly_plan_create_shared"
        call(fn, ctypes.byref(self.desc), _lib.dbl_array(self.wavelengths), self.max_objects,
             ctypes.byref(self.handle))
        self.gemm_pair, self.split_k = gemm_pair, bool(split_k)
        if gemm_pair is not None or not split_k:
            call("dlx_poly_plan_set_gemm_form", self.handle,
                 0 if gemm_pair is None else (2 if gemm_pair else 1), int(bool(split_k)))

    def workspace_bytes(self) -> int:
        n = ctypes.c_size_t(0)
        call("dlx_poly_workspace_bytes", ctypes.byref(self.desc), self.max_objects,
             ctypes.byref(n))
        return int(n.value)

    def attach_workspace(self, ws: torch.Tensor) -> None:
        """Use ``ws`` (a 256-byte aligned uint8 CUDA tensor) for the per-call buffers."""
        call("dlx_poly_attach_workspace", self.handle, ptr(ws), ws.numel() * ws.element_size())

    # ---- batched objects (requests or point sources) ----
    _OBJ_FIELDS = ("amp", "amp_scale", "opd", "phase", "weights", "psf", "g_psf", "g_amp",
                   "g_opd", "g_phase", "g_w", "g_tilt")

    @classmethod
    def _object_array(cls, objs):
        arr = (_lib.PolyObject * max(1, len(objs)))()
        for i, o in enumerate(objs):
            for f in cls._OBJ_FIELDS:
                t = o.get(f)
                setattr(arr[i], f, ptr(t.contiguous() if t is not None else None))
            tilt = o.get("tilt", (0.0, 0.0))
            arr[i].tilt_x, arr[i].tilt_y = float(tilt[0]), float(tilt[1])
        return arr

    def forward_objects(self, objs, psf_sum=None, accumulate=False):
        """PSFs of several objects: dicts with amp/amp_scale/opd/phase/weights/tilt/psf."""
        arr = self._object_array(objs)
        call("dlx_poly_forward", self.handle, ctypes.cast(arr, ctypes.c_void_p), len(objs),
             ptr(psf_sum), int(bool(accumulate)), _stream())

    def forward_backward_objects(self, objs):
        """PSF and reverse pass in one sweep; every object needs its cotangent g_psf."""
        arr = self._object_array(objs)
        call("dlx_poly_forward_backward", self.handle, ctypes.cast(arr, ctypes.c_void_p),
             len(objs), _stream())

    def backward_objects(self, objs, sum_grads=None):
        """Reverse pass; ``sum_grads`` ({"amp","opd","phase"} tensors) sums pixel gradients."""
        arr = self._object_array(objs)
        if sum_grads is None:
            call("dlx_poly_backward", self.handle, ctypes.cast(arr, ctypes.c_void_p), len(objs),
                 _stream())
        else:
            call("dlx_poly_backward_sum", self.handle, ctypes.cast(arr, ctypes.c_void_p),
                 len(objs), ptr(sum_grads.get("amp")), ptr(sum_grads.get("opd")),
                 ptr(sum_grads.get("phase")), _stream())

    @property
    def footprint(self) -> int:
        n = ctypes.c_size_t(0)
        call("dlx_poly_plan_footprint", self.handle, ctypes.byref(n))
        return int(n.value)

    def tilt_basis(self):
        """[2, N, N] pupil coordinates (X, Y) in metres, cached on the device."""
        tb = getattr(self, "_tilt_basis", None)
        if tb is None:
            n = self.n_in
            xs = (torch.arange(n, dtype=torch.float64) - (n - 1) / 2) * self.pixel_scale_in
            yy, xx = torch.meshgrid(xs, xs, indexing="ij")
            tb = torch.stack([xx, yy]).to(device="cuda", dtype=torch.float32).contiguous()
            self._tilt_basis = tb
        return tb

    def psf(self, amp, amp_scale, opd, phase, weights, tilt=(0.0, 0.0), out=None, keep=False):
        """PSF of one object. ``keep``: also keep the focal fields, so that a
        reverse pass reusing this forward (grad with its forward_token()) skips
        recomputing them."""
        amp, amp_scale, opd, phase, weights = map(_contig, (amp, amp_scale, opd, phase, weights))
        dev = weights.device
        if out is None:
            out = torch.empty((self.n_out, self.n_out), dtype=torch.float32, device=dev)
        if keep:
            call("dlx_poly_keep_focal", self.handle, 1)
        call("dlx_poly_psf", self.handle, ptr(amp), ptr(amp_scale), ptr(opd), ptr(phase),
             ptr(weights), float(tilt[0]), float(tilt[1]), ptr(out), _stream())
        return out

    def forward_token(self) -> int:
        """Token of the forward state the workspace still holds (0 if none)."""
        t = ctypes.c_ulonglong(0)
        call("dlx_poly_forward_token", self.handle, ctypes.byref(t))
        return int(t.value)

    def grad(self, amp, amp_scale, opd, phase, weights, g_psf, tilt=(0.0, 0.0),
             want=("amp", "opd", "phase", "w"), reuse_token=0):
        """Reverse pass. ``reuse_token`` (from forward_token() after the matching
        psf call) lets it start from that forward's workspace when the plan has
        not been used since; otherwise everything is recomputed."""
        amp, amp_scale, opd, phase, weights = map(_contig, (amp, amp_scale, opd, phase, weights))
        dev = g_psf.device
        n = self.n_in
        g_amp = torch.empty((n, n), dtype=torch.float32, device=dev) if "amp" in want else None
        g_opd = torch.empty((n, n), dtype=torch.float32, device=dev) if "opd" in want else None
        g_ph = torch.empty((n, n), dtype=torch.float32, device=dev) if "phase" in want else None
        g_w = (torch.empty((len(self.wavelengths),), dtype=torch.float32, device=dev)
               if "w" in want else None)
        if reuse_token:
            call("dlx_poly_reuse_forward", self.handle, ctypes.c_ulonglong(reuse_token))
        call("dlx_poly_psf_grad", self.handle, ptr(amp), ptr(amp_scale), ptr(opd), ptr(phase),
             ptr(weights), float(tilt[0]), float(tilt[1]), ptr(g_psf.contiguous()), ptr(g_amp),
             ptr(g_opd), ptr(g_ph), ptr(g_w), _stream())
        return {"amp": g_amp, "opd": g_opd, "phase": g_ph, "w": g_w}


class ScenePlan(_Plan):
    """Many point sources through one pupil: per-source tilt as a DFT output shift."""

    _destroy = "dlx_scene_plan_destroy"

    def __init__(self, wavelengths, n_in, pixel_scale_in, n_out, pixel_scale_out,
                 focal_length=None, variant=None, max_sources=32):
        super().__init__()
        _lib.require_cuda()
        self.wavelengths = tuple(float(w) for w in wavelengths)
        self.n_in, self.n_out = int(n_in), int(n_out)
        self.variant = resolve_variant(self.n_in, self.n_out, variant)
        self.desc = _lib.SceneDesc(len(self.wavelengths), self.n_in, self.n_out,
                                   float(pixel_scale_in), float(pixel_scale_out),
                                   float(focal_length) if focal_length is not None else 0.0,
                                   self.variant, int(max_sources))
        call("dlx_scene_plan_create", ctypes.byref(self.desc), _lib.dbl_array(self.wavelengths),
             ctypes.byref(self.handle))

    @property
    def footprint(self) -> int:
        n = ctypes.c_size_t(0)
        call("dlx_scene_plan_footprint", self.handle, ctypes.byref(n))
        return int(n.value)

    def forward(self, amp, amp_scale, opd, phase, positions, weights, out=None):
        """Summed image of sources at positions [S, 2] (rad, float64) with weights [S, L]."""
        positions = positions.to(device="cuda", dtype=torch.float64).contiguous()
        weights = weights.to(device="cuda", dtype=torch.float32).contiguous()
        S = positions.shape[0]
        if out is None:
            out = torch.empty((self.n_out, self.n_out), dtype=torch.float32, device="cuda")
        call("dlx_scene_forward", self.handle, ptr(_contig(amp)), ptr(amp_scale),
             ptr(_contig(opd)), ptr(_contig(phase)), ptr(positions), ptr(weights), S, ptr(out), 0,
             _stream())
        return out

    def forward_token(self) -> int:
        """Token of the retained forward state (0 if none)."""
        t = ctypes.c_ulonglong(0)
        call("dlx_scene_forward_token", self.handle, ctypes.byref(t))
        return int(t.value)

    def set_retain_limit(self, nbytes: int) -> None:
        """Cap (bytes) on the fields a forward keeps for its backward; 0 disables."""
        call("dlx_scene_set_retain_limit", self.handle, int(nbytes))

    def backward(self, amp, amp_scale, opd, phase, positions, weights, g_image, want_pos=True,
                 want_w=True, reuse_token=0):
        """Reverse pass. ``reuse_token`` (forward_token() after the matching
        forward) lets it start from the retained fields when they are intact."""
        positions = positions.to(device="cuda", dtype=torch.float64).contiguous()
        weights = weights.to(device="cuda", dtype=torch.float32).contiguous()
        S = positions.shape[0]
        if reuse_token:
            call("dlx_scene_reuse_forward", self.handle, ctypes.c_ulonglong(reuse_token))
        g_pos = torch.empty((S, 2), dtype=torch.float32, device="cuda") if want_pos else None
        g_w = torch.empty(weights.shape, dtype=torch.float32, device="cuda") if want_w else None
        call("dlx_scene_backward", self.handle, ptr(_contig(amp)), ptr(amp_scale),
             ptr(_contig(opd)), ptr(_contig(phase)), ptr(positions), ptr(weights), S,
             ptr(g_image.contiguous()), ptr(g_pos), ptr(g_w), _stream())
        return g_pos, g_w


APERTURE_SHAPES = {"circle": 0, "square": 1, "rectangle": 2, "polygon": 3}


def aperture_desc(npixels, pixel_scale, radius, softening=1.0, occulting=False,
                  translation=None, rotation=None, compression=None, shear=None,
                  shape="circle", width=0.0, height=0.0, nsides=0):
    """dlx_aperture_desc of a dynamic aperture under a CoordTransform: a circle of
    `radius`, a square of side `width`, a `width` x `height` rectangle, or a regular
    polygon of `nsides` with circumradius `radius`."""
    d = _lib.ApertureDesc()
    d.shape = APERTURE_SHAPES[shape]
    d.width, d.height, d.nsides = float(width), float(height), int(nsides)
    d.npixels = int(npixels)
    d.pixel_scale = float(pixel_scale)
    t = (0.0, 0.0) if translation is None else tuple(float(v) for v in translation)
    c = (1.0, 1.0) if compression is None else tuple(float(v) for v in compression)
    sh = (0.0, 0.0) if shear is None else tuple(float(v) for v in shear)
    d.translation[0], d.translation[1] = t
    d.compression[0], d.compression[1] = c
    d.shear[0], d.shear[1] = sh
    d.rotation = 0.0 if rotation is None else float(rotation)
    d.radius = float(radius)
    d.softening = float(softening)
    d.occulting = int(bool(occulting))
    return d


def _noll_array(noll):
    arr = (ctypes.c_int * max(1, len(noll)))(*[int(j) for j in noll])
    return arr


def aberrated_aperture(desc, noll, coeffs, want_trans=True, want_opd=True):
    """(transmission, opd) [N, N] of a dynamic aperture; either may be skipped (None)."""
    dev = _lib.require_cuda()
    n = desc.npixels
    trans = torch.empty((n, n), dtype=torch.float32, device=dev) if want_trans else None
    opd = torch.empty((n, n), dtype=torch.float32, device=dev) if want_opd else None
    c = None if coeffs is None else _f32(coeffs, dev)
    call("dlx_aberrated_aperture", ctypes.byref(desc), _noll_array(noll), len(noll), ptr(c),
         ptr(trans), ptr(opd), _stream())
    return trans, opd


def aberrated_aperture_grad(desc, noll, g_opd):
    """d<g_opd, opd>/d coefficients [K]."""
    dev = g_opd.device
    g = torch.empty((len(noll),), dtype=torch.float32, device=dev)
    call("dlx_aberrated_aperture_grad", ctypes.byref(desc), _noll_array(noll), len(noll),
         ptr(g_opd.contiguous()), ptr(g), _stream())
    return g


def conv2d_same(x, kernel):
    """[..., H, W] images convolved with a [K0, K1] kernel, mode "same"."""
    x = _contig(x)
    k = _contig(kernel.to(device=x.device, dtype=torch.float32))
    H, W = x.shape[-2:]
    B = x.numel() // (H * W)
    out = torch.empty_like(x)
    call("dlx_conv2d_same", ptr(x), B, H, W, ptr(k), k.shape[0], k.shape[1], ptr(out), _stream())
    return out


def conv2d_same_backward(x, kernel, g, want_x=True, want_k=True):
    x = _contig(x)
    k = _contig(kernel.to(device=x.device, dtype=torch.float32))
    g = _contig(g)
    H, W = x.shape[-2:]
    B = x.numel() // (H * W)
    gx = torch.empty_like(x) if want_x else None
    gk = torch.empty_like(k) if want_k else None
    call("dlx_conv2d_same_backward", ptr(x), B, H, W, ptr(k), k.shape[0], k.shape[1], ptr(g),
         ptr(gx), ptr(gk), _stream())
    return gx, gk


mft_plans = _PlanCache(16)
fft_plans = _PlanCache(8)
poly_plans = _PlanCache(8)
scene_plans = _PlanCache(4)
xform_plans = _PlanCache(8)  # ABCD propagators: LCT transforms and ASM plans


def get_mft_plan(wavelengths, n_in, pixel_scale_in, n_out, pixel_scale_out, focal_length=None,
                 shift=(0.0, 0.0), inverse=False, variant=None):
    wl = tuple(float(w) for w in wavelengths)
    v = resolve_variant(n_in, n_out, variant)
    key = (wl, int(n_in), float(pixel_scale_in), int(n_out), float(pixel_scale_out),
           None if focal_length is None else float(focal_length),
           (float(shift[0]), float(shift[1])), bool(inverse), v)
    return mft_plans.get(key, lambda: MFTPlan(wl, n_in, pixel_scale_in, n_out, pixel_scale_out,
                                              focal_length, shift, inverse,
                                              "fp32" if v == 0 else "split_bf16"))


def get_fft_plan(wavelengths, n_in, pixel_scale_in, pad=2, focal_length=None, inverse=False,
                 ramps=None, variant=None):
    wl = tuple(float(w) for w in wavelengths)
    v = resolve_fft_variant(n_in, pad, variant)
    key = (wl, int(n_in), float(pixel_scale_in), int(pad),
           None if focal_length is None else float(focal_length), bool(inverse),
           None if ramps is None else (float(ramps[0]), float(ramps[1])), v)
    return fft_plans.get(key, lambda: FFTPlan(wl, n_in, pixel_scale_in, pad, focal_length,
                                              inverse, ramps, v))


def get_scene_plan(wavelengths, n_in, pixel_scale_in, n_out, pixel_scale_out,
                   focal_length=None, variant=None, max_sources=32):
    wl = tuple(float(w) for w in wavelengths)
    v = resolve_variant(n_in, n_out, variant)
    key = (wl, int(n_in), float(pixel_scale_in), int(n_out), float(pixel_scale_out),
           None if focal_length is None else float(focal_length), v, int(max_sources),
           torch.cuda.current_device())
    return scene_plans.get(key, lambda: ScenePlan(wl, n_in, pixel_scale_in, n_out, pixel_scale_out,
                                                  focal_length, v, max_sources))


def get_poly_plan(wavelengths, n_in, pixel_scale_in, n_out, pixel_scale_out, focal_length=None,
                  variant=None, max_objects=1):
    wl = tuple(float(w) for w in wavelengths)
    v = resolve_variant(n_in, n_out, variant)
    key = (wl, int(n_in), float(pixel_scale_in), int(n_out), float(pixel_scale_out),
           None if focal_length is None else float(focal_length), v, int(max_objects))
    return poly_plans.get(key, lambda: PolyPlan(wl, n_in, pixel_scale_in, n_out, pixel_scale_out,
                                                focal_length,
                                                "fp32" if v == 0 else "split_bf16",
                                                max_objects))


# ---------------------------------------------------------------------------
# Elementwise and reductions
# ---------------------------------------------------------------------------
def phasor(wavelengths, n, pixel_scale, field=None, amp=None, opd=None, phase=None,
           amp_scale=None, weights=None, const_scale=1.0, tilt=(0.0, 0.0), out=None):
    """field * amp * exp(i (2 pi (opd + tilt . xy) / lambda + phase)) for every wavelength."""
    dev = _lib.require_cuda()
    wl = [float(w) for w in torch.as_tensor(wavelengths, dtype=torch.float64).reshape(-1)]
    b = len(wl)
    if out is None:
        out = torch.empty((b, n, n), dtype=torch.complex64, device=dev)
    call("dlx_phasor", ptr(field), ptr(amp), ptr(opd), ptr(phase), ptr(amp_scale), ptr(weights),
         float(const_scale), _lib.dbl_array(wl), b, int(n), float(pixel_scale), float(tilt[0]),
         float(tilt[1]), ptr(out), _stream())
    return out


def power_scale(field, value=1.0):
    """sqrt(value / sum |E|^2) per batch element (Wavefront.normalise, mode "power")."""
    f = field.reshape(-1, field.shape[-2], field.shape[-1]).contiguous()
    out = torch.empty((f.shape[0],), dtype=torch.float32, device=f.device)
    call("dlx_power_scale", ptr(f), f.shape[0], f.shape[-1], float(value), ptr(out), _stream())
    return out


def amp_norm(amp, value=1.0, out=None):
    if out is None:
        out = torch.empty((), dtype=torch.float32, device=amp.device)
    call("dlx_amp_norm", ptr(amp.contiguous()), amp.shape[-1], float(value), ptr(out), _stream())
    return out


_side_streams = {}


def _side_stream(device):
    s = _side_streams.get(device)
    if s is None:
        s = _side_streams[device] = torch.cuda.Stream(device=device)
    return s


class AmpNormFork:
    """amp_norm on a side stream forked from the current one, so that it runs
    beside the work issued next on the current stream; ``join()`` makes the
    current stream wait for it and returns the scale. The scale tensor is
    allocated on the current stream and the amplitude stays referenced, so
    neither memory is reused before the join (under CUDA-graph capture the
    fork and the join become a branch of the graph)."""

    def __init__(self, amp, value=1.0):
        self.amp = amp.contiguous()
        self.cur = torch.cuda.current_stream(amp.device)
        self.side = _side_stream(amp.device)
        self.scale = torch.empty((), dtype=torch.float32, device=amp.device)
        self.side.wait_stream(self.cur)
        with torch.cuda.stream(self.side):
            amp_norm(self.amp, value, out=self.scale)

    def join(self):
        self.cur.wait_stream(self.side)
        return self.scale


def amp_norm_backward(amp, g_eff, value=1.0):
    out = torch.empty_like(amp)
    call("dlx_amp_norm_backward", ptr(amp.contiguous()), ptr(g_eff.contiguous()), amp.shape[-1],
         float(value), ptr(out), _stream())
    return out


def basis_eval(basis, coeffs, base=None):
    """sum_k coeffs[k] basis[k] (+ base) over flattened coefficient dims (utils/math.py:177-196)."""
    k = coeffs.numel()
    spatial = basis.shape[coeffs.dim():]
    npix = int(math.prod(spatial))
    out = torch.empty(spatial, dtype=torch.float32, device=basis.device)
    call("dlx_basis_eval", ptr(basis.contiguous()), ptr(coeffs.contiguous().float()),
         ptr(base), k, npix, ptr(out), _stream())
    return out


def basis_grad(basis, g, coeff_shape):
    k = int(math.prod(coeff_shape))
    out = torch.empty(coeff_shape, dtype=torch.float32, device=basis.device)
    call("dlx_basis_grad", ptr(basis.contiguous()), ptr(g.contiguous()), k, g.numel(), ptr(out),
         _stream())
    return out


def psf_sum(field):
    f = field.reshape(-1, field.shape[-2], field.shape[-1]).contiguous()
    out = torch.empty(f.shape[-2:], dtype=torch.float32, device=f.device)
    call("dlx_psf_sum", ptr(f), f.shape[0], f.shape[-1] * f.shape[-2], ptr(out), _stream())
    return out


def psf_sum_weighted(field, weights=None):
    """sum_b w_b |field_b|^2 of [B, N, N] focal fields (weights None: 1)."""
    f = field.reshape(-1, field.shape[-2], field.shape[-1]).contiguous()
    w = None if weights is None else weights.to(device=f.device, dtype=torch.float32).contiguous()
    out = torch.empty(f.shape[-2:], dtype=torch.float32, device=f.device)
    call("dlx_psf_sum_weighted", ptr(f), ptr(w), f.shape[0], f.shape[-1] * f.shape[-2],
         ptr(out), _stream())
    return out


def psf_sum_weighted_backward(field, weights, g, want_field=True, want_weights=True):
    f = field.reshape(-1, field.shape[-2], field.shape[-1]).contiguous()
    w = None if weights is None else weights.to(device=f.device, dtype=torch.float32).contiguous()
    gf = torch.empty_like(f) if want_field else None
    gw = torch.empty((f.shape[0],), dtype=torch.float32, device=f.device) if want_weights \
        else None
    call("dlx_psf_sum_weighted_backward", ptr(f), ptr(w), f.shape[0],
         f.shape[-1] * f.shape[-2], ptr(g.contiguous()), ptr(gf), ptr(gw), _stream())
    return gf, gw


def phasor_backward(wavelengths, field, amp, opd, phase, g, want_field=True, want_amp=True,
                    want_opd=True, want_phase=True):
    """Reverse pass of the phasor multiply (see dlx_phasor_backward)."""
    wl = [float(w) for w in torch.as_tensor(wavelengths, dtype=torch.float64).reshape(-1)]
    gg = g.contiguous()
    n = gg.shape[-1]
    pix = (n, n)
    dev = gg.device
    gf = torch.empty_like(gg) if want_field else None
    g_amp = torch.empty(pix, dtype=torch.float32, device=dev) if want_amp else None
    g_opd = torch.empty(pix, dtype=torch.float32, device=dev) if want_opd else None
    g_ph = torch.empty(pix, dtype=torch.float32, device=dev) if want_phase else None
    call("dlx_phasor_backward", ptr(field), ptr(amp), ptr(opd), ptr(phase),
         _lib.dbl_array(wl), len(wl), n, ptr(gg), ptr(gf), ptr(g_amp), ptr(g_opd), ptr(g_ph),
         _stream())
    return gf, g_amp, g_opd, g_ph


_NORM_MODES = {"power": 0, "peak": 1}


def normalise(field, mode="power", value=1.0):
    """Each [N, N] plane of `field` scaled to unit power or unit peak (times value)."""
    if mode not in _NORM_MODES:
        raise ValueError("mode must be 'power' or 'peak'")
    f = field.reshape(-1, field.shape[-2], field.shape[-1]).contiguous()
    out = torch.empty_like(f)
    call("dlx_normalise", ptr(f), f.shape[0], f.shape[-1] * f.shape[-2], _NORM_MODES[mode],
         float(value), ptr(out), None, _stream())
    return out.reshape(field.shape)


def normalise_backward(field, g, mode="power", value=1.0):
    f = field.reshape(-1, field.shape[-2], field.shape[-1]).contiguous()
    gg = g.reshape(f.shape).contiguous()
    gin = torch.empty_like(f)
    call("dlx_normalise_backward", ptr(f), f.shape[0], f.shape[-1] * f.shape[-2],
         _NORM_MODES[mode], float(value), ptr(gg), ptr(gin), _stream())
    return gin.reshape(field.shape)


def downsample(psf, k, mean=False, flat=None):
    n = psf.shape[-1]
    if psf.shape[-2] != n:
        raise ValueError(f"Input array has shape {tuple(psf.shape)}, which is not square")
    if n % k != 0:
        raise ValueError(f"Input array has {n} pixels, which is not divisible by {k}")
    out = torch.empty((n // k, n // k), dtype=torch.float32, device=psf.device)
    call("dlx_downsample", ptr(psf.contiguous()), n, int(k), int(bool(mean)), ptr(flat), ptr(out),
         _stream())
    return out


def downsample_backward(psf, g_out, k, mean=False, flat=None, want_flat=False):
    n = psf.shape[-1]
    g_in = torch.empty((n, n), dtype=torch.float32, device=g_out.device)
    g_flat = torch.empty_like(g_out) if want_flat else None
    call("dlx_downsample_backward", ptr(psf.contiguous()), ptr(g_out.contiguous()), n, int(k),
         int(bool(mean)), ptr(flat), ptr(g_in), ptr(g_flat), _stream())
    return g_in, g_flat
