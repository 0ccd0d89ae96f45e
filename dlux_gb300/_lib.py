"""ctypes binding of ``libdluxgb.so`` (the C ABI in ``include/dluxgb.h``).

The library is the only compute path of this package: if it cannot be loaded,
or no CUDA device is present, every operation raises instead of computing
anything on the host.
"""

from __future__ import annotations

import ctypes
import os
import threading
from pathlib import Path

import torch

_LIB_PATH = Path(__file__).resolve().parent / "libdluxgb.so"
_lock = threading.Lock()
_lib = None

DLX_OK = 0
DLX_ERR_ARG = 1
DLX_ERR_SHAPE = 2
DLX_ERR_NOMEM = 3
DLX_ERR_CUDA = 4
DLX_ERR_TIMEOUT = 5
DLX_ERR_UNSUPPORTED = 6

VARIANT_FP32 = 0
VARIANT_SPLIT_BF16 = 1
VARIANT_RADIX = 2          # FFT plans only: radix-2 line FFTs

_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_c_vp = ctypes.c_void_p
_c_ll = ctypes.c_longlong


class MftDesc(ctypes.Structure):
    _fields_ = [
        ("batch", _c_int), ("n_in", _c_int), ("n_out", _c_int),
        ("pixel_scale_in", _c_dbl), ("pixel_scale_out", _c_dbl), ("focal_length", _c_dbl),
        ("shift_x", _c_dbl), ("shift_y", _c_dbl), ("inverse", _c_int), ("variant", _c_int),
    ]


class XformAxis(ctypes.Structure):
    _fields_ = [
        ("a_in", _c_dbl), ("b_in", _c_dbl), ("a_out", _c_dbl), ("b_out", _c_dbl),
        ("sigma", _c_dbl), ("q_in", _c_dbl), ("q_out", _c_dbl), ("phase", _c_dbl),
        ("scale", _c_dbl),
    ]


class XformDesc(ctypes.Structure):
    _fields_ = [("batch", _c_int), ("n_in", _c_int), ("n_out", _c_int), ("variant", _c_int)]


class AsmDesc(ctypes.Structure):
    _fields_ = [
        ("batch", _c_int), ("n_in", _c_int), ("n_pad", _c_int),
        ("pixel_scale", _c_dbl), ("distance", _c_dbl), ("variant", _c_int),
    ]


class FftDesc(ctypes.Structure):
    _fields_ = [
        ("batch", _c_int), ("n_in", _c_int), ("pad", _c_int),
        ("pixel_scale_in", _c_dbl), ("focal_length", _c_dbl), ("inverse", _c_int),
        ("apply_ramps", _c_int), ("center_in", _c_dbl), ("center_out", _c_dbl),
        ("variant", _c_int),
    ]


class PolyDesc(ctypes.Structure):
    _fields_ = [
        ("n_wavelengths", _c_int), ("n_in", _c_int), ("n_out", _c_int),
        ("pixel_scale_in", _c_dbl), ("pixel_scale_out", _c_dbl), ("focal_length", _c_dbl),
        ("variant", _c_int), ("operand_mode", _c_int),
    ]


class PolyObject(ctypes.Structure):
    """dlx_poly_object: one request or source of a batched PSF evaluation."""
    _fields_ = [
        ("amp", _c_vp), ("amp_scale", _c_vp), ("opd", _c_vp), ("phase", _c_vp),
        ("weights", _c_vp), ("tilt_x", _c_dbl), ("tilt_y", _c_dbl), ("psf", _c_vp),
        ("g_psf", _c_vp), ("g_amp", _c_vp), ("g_opd", _c_vp), ("g_phase", _c_vp),
        ("g_w", _c_vp), ("g_tilt", _c_vp),
    ]


class ApertureDesc(ctypes.Structure):
    """dlx_aperture_desc: a dynamic aperture and its coordinate transformation."""
    _fields_ = [
        ("npixels", _c_int), ("pixel_scale", _c_dbl), ("translation", _c_dbl * 2),
        ("rotation", _c_dbl), ("compression", _c_dbl * 2), ("shear", _c_dbl * 2),
        ("radius", _c_dbl), ("softening", _c_dbl), ("occulting", _c_int),
        ("shape", _c_int), ("width", _c_dbl), ("height", _c_dbl), ("nsides", _c_int),
    ]


class SceneDesc(ctypes.Structure):
    _fields_ = [
        ("n_wavelengths", _c_int), ("n_in", _c_int), ("n_out", _c_int),
        ("pixel_scale_in", _c_dbl), ("pixel_scale_out", _c_dbl), ("focal_length", _c_dbl),
        ("variant", _c_int), ("max_sources", _c_int),
    ]


class ServeBatch(ctypes.Structure):
    """dlx_serve_batch: one batch of serving requests that share a plan."""
    _fields_ = [
        ("n_objects", _c_int), ("n_grad", _c_int), ("n_coeffs", _c_int),
        ("basis", _c_vp), ("amp", _c_vp), ("amp_scale", _c_vp),
        ("h_coeffs", _c_vp), ("h_weights", _c_vp), ("h_g_psf", _c_vp), ("h_psf", _c_vp),
        ("h_grad", _c_vp), ("d_work", _c_vp), ("d_work_bytes", ctypes.c_size_t),
    ]


_SIGNATURES = {
    "dlx_last_error": (ctypes.c_char_p, []),
    "dlx_version": (_c_int, []),
    "dlx_device_status": (_c_int, [_c_vp, ctypes.POINTER(_c_int)]),
    "dlx_launch_count": (_c_ll, []),
    "dlx_gemm_timing_begin": (_c_int, []),
    "dlx_gemm_timing_end": (_c_int, [ctypes.POINTER(_c_dbl), ctypes.POINTER(_c_int),
                                     ctypes.POINTER(_c_dbl)]),
    "dlx_transfer_matrix": (_c_int, [_c_vp, _c_int, _c_int, _c_dbl, _c_int, _c_dbl, _c_dbl,
                                     _c_dbl, _c_int, _c_int, _c_vp, _c_vp]),
    "dlx_mft_plan_create": (_c_int, [ctypes.POINTER(MftDesc), _c_vp, ctypes.POINTER(_c_vp)]),
    "dlx_xform_plan_create": (_c_int, [ctypes.POINTER(XformDesc), _c_vp, _c_vp,
                                       ctypes.POINTER(_c_vp)]),
    "dlx_xform_plan_destroy": (_c_int, [_c_vp]),
    "dlx_xform_forward": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_xform_adjoint": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_asm_plan_create": (_c_int, [ctypes.POINTER(AsmDesc), _c_vp, ctypes.POINTER(_c_vp)]),
    "dlx_asm_plan_destroy": (_c_int, [_c_vp]),
    "dlx_asm_forward": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_asm_adjoint": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_mft_plan_destroy": (_c_int, [_c_vp]),
    "dlx_mft_forward": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_mft_adjoint": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_mft_forward_noalloc": (_c_int, [_c_vp, _c_int, _c_int, _c_dbl, _c_int, _c_dbl, _c_vp,
                                         _c_dbl, _c_dbl, _c_dbl, _c_int, _c_vp, _c_vp]),
    "dlx_fft_plan_create": (_c_int, [ctypes.POINTER(FftDesc), _c_vp, ctypes.POINTER(_c_vp)]),
    "dlx_fft_plan_destroy": (_c_int, [_c_vp]),
    "dlx_fft_forward": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_fft_adjoint": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_phasor": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_dbl, _c_vp, _c_int,
                            _c_int, _c_dbl, _c_dbl, _c_dbl, _c_vp, _c_vp]),
    "dlx_power_scale": (_c_int, [_c_vp, _c_int, _c_int, _c_dbl, _c_vp, _c_vp]),
    "dlx_amp_norm": (_c_int, [_c_vp, _c_int, _c_dbl, _c_vp, _c_vp]),
    "dlx_amp_norm_backward": (_c_int, [_c_vp, _c_vp, _c_int, _c_dbl, _c_vp, _c_vp]),
    "dlx_basis_eval": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int, _c_ll, _c_vp, _c_vp]),
    "dlx_basis_grad": (_c_int, [_c_vp, _c_vp, _c_int, _c_ll, _c_vp, _c_vp]),
    "dlx_psf_sum": (_c_int, [_c_vp, _c_int, _c_ll, _c_vp, _c_vp]),
    "dlx_psf_sum_weighted": (_c_int, [_c_vp, _c_vp, _c_int, _c_ll, _c_vp, _c_vp]),
    "dlx_psf_sum_weighted_backward": (_c_int, [_c_vp, _c_vp, _c_int, _c_ll, _c_vp, _c_vp,
                                               _c_vp, _c_vp]),
    "dlx_phasor_backward": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_int, _c_int, _c_vp,
                                     _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_normalise": (_c_int, [_c_vp, _c_int, _c_ll, _c_int, _c_dbl, _c_vp, _c_vp, _c_vp]),
    "dlx_normalise_backward": (_c_int, [_c_vp, _c_int, _c_ll, _c_int, _c_dbl, _c_vp, _c_vp,
                                        _c_vp]),
    "dlx_downsample": (_c_int, [_c_vp, _c_int, _c_int, _c_int, _c_vp, _c_vp, _c_vp]),
    "dlx_downsample_backward": (_c_int, [_c_vp, _c_vp, _c_int, _c_int, _c_int, _c_vp, _c_vp,
                                         _c_vp, _c_vp]),
    "dlx_poly_plan_create": (_c_int, [ctypes.POINTER(PolyDesc), _c_vp, ctypes.POINTER(_c_vp)]),
    "dlx_poly_plan_create_batched": (_c_int, [ctypes.POINTER(PolyDesc), _c_vp, _c_int,
                                              ctypes.POINTER(_c_vp)]),
    "dlx_poly_plan_create_shared": (_c_int, [ctypes.POINTER(PolyDesc), _c_vp, _c_int,
                                             ctypes.POINTER(_c_vp)]),
    "dlx_poly_workspace_bytes": (_c_int, [ctypes.POINTER(PolyDesc), _c_int,
                                          ctypes.POINTER(ctypes.c_size_t)]),
    "dlx_poly_attach_workspace": (_c_int, [_c_vp, _c_vp, ctypes.c_size_t]),
    "dlx_poly_forward": (_c_int, [_c_vp, _c_vp, _c_int, _c_vp, _c_int, _c_vp]),
    "dlx_poly_backward": (_c_int, [_c_vp, _c_vp, _c_int, _c_vp]),
    "dlx_poly_forward_token": (_c_int, [_c_vp, ctypes.POINTER(ctypes.c_ulonglong)]),
    "dlx_poly_keep_focal": (_c_int, [_c_vp, _c_int]),
    "dlx_poly_reuse_forward": (_c_int, [_c_vp, ctypes.c_ulonglong]),
    "dlx_set_split_k": (_c_int, [_c_int]),
    "dlx_set_gemm_pair": (_c_int, [_c_int]),
    "dlx_gemm_pair_clusters": (_c_int, [ctypes.POINTER(_c_int)]),
    "dlx_set_wait_limit_ns": (_c_int, [ctypes.c_ulonglong]),
    "dlx_poly_plan_set_gemm_form": (_c_int, [_c_vp, _c_int, _c_int]),
    "dlx_test_gemm_withhold_copies": (_c_int, [_c_int]),
    "dlx_scene_forward_token": (_c_int, [_c_vp, ctypes.POINTER(ctypes.c_ulonglong)]),
    "dlx_scene_reuse_forward": (_c_int, [_c_vp, ctypes.c_ulonglong]),
    "dlx_scene_set_retain_limit": (_c_int, [_c_vp, ctypes.c_size_t]),
    "dlx_poly_forward_backward": (_c_int, [_c_vp, _c_vp, _c_int, _c_vp]),
    "dlx_poly_backward_sum": (_c_int, [_c_vp, _c_vp, _c_int, _c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_poly_plan_destroy": (_c_int, [_c_vp]),
    "dlx_poly_plan_footprint": (_c_int, [_c_vp, ctypes.POINTER(ctypes.c_size_t)]),
    "dlx_poly_plan_info": (_c_int, [_c_vp, ctypes.POINTER(_c_int), ctypes.POINTER(_c_int),
                                    ctypes.POINTER(_c_int), ctypes.POINTER(_c_int)]),
    "dlx_conv2d_same": (_c_int, [_c_vp, _c_int, _c_int, _c_int, _c_vp, _c_int, _c_int, _c_vp,
                                 _c_vp]),
    "dlx_conv2d_same_backward": (_c_int, [_c_vp, _c_int, _c_int, _c_int, _c_vp, _c_int, _c_int,
                                          _c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_zernike_table": (_c_int, [_c_vp, _c_int, _c_vp, _c_vp, _c_vp]),
    "dlx_aberrated_aperture": (_c_int, [ctypes.POINTER(ApertureDesc), _c_vp, _c_int, _c_vp,
                                        _c_vp, _c_vp, _c_vp]),
    "dlx_aberrated_aperture_grad": (_c_int, [ctypes.POINTER(ApertureDesc), _c_vp, _c_int,
                                             _c_vp, _c_vp, _c_vp]),
    "dlx_scene_plan_create": (_c_int, [ctypes.POINTER(SceneDesc), _c_vp, ctypes.POINTER(_c_vp)]),
    "dlx_scene_plan_destroy": (_c_int, [_c_vp]),
    "dlx_scene_plan_footprint": (_c_int, [_c_vp, ctypes.POINTER(ctypes.c_size_t)]),
    "dlx_scene_forward": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_int, _c_vp,
                                   _c_int, _c_vp]),
    "dlx_scene_backward": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_int,
                                    _c_vp, _c_vp, _c_vp, _c_vp]),
    "dlx_serve_workspace_bytes": (_c_int, [_c_int, _c_int, _c_int, _c_int, _c_int,
                                           ctypes.POINTER(ctypes.c_size_t)]),
    "dlx_serve_run": (_c_int, [_c_vp, ctypes.POINTER(ServeBatch), _c_vp]),
    "dlx_poly_psf": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_dbl, _c_dbl, _c_vp,
                              _c_vp]),
    "dlx_poly_psf_grad": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_dbl, _c_dbl,
                                   _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
}


def exported_symbols():
    """Names of the C entry points this binding declares."""
    return list(_SIGNATURES)


def load(path: str | os.PathLike | None = None):
    """Load (once) and return the ctypes library handle; raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else _LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"dlux_gb300 CUDA library not found at {p}; build it with "
                "`python -m dlux_gb300._build` (nvcc, sm_103a)")
        lib = ctypes.CDLL(str(p))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


class DluxError(RuntimeError):
    """A failing C-ABI call (CUDA error, allocation failure, timeout)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[dlux status {code}] {msg}")
        self.code = code


def check(status: int) -> None:
    """Map a DLX status to dLux's Python exceptions."""
    if status == DLX_OK:
        return
    msg = load().dlx_last_error().decode(errors="replace")
    if status in (DLX_ERR_ARG, DLX_ERR_SHAPE):
        raise ValueError(msg)
    raise DluxError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def stream_ptr(device=None) -> int:
    """Raw handle of torch's current CUDA stream."""
    return torch.cuda.current_stream(device).cuda_stream


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("dlux_gb300 needs a CUDA device (GB300, sm_103a); none is visible")
    load()
    return torch.device("cuda", torch.cuda.current_device())


def ptr(t) -> int | None:
    """Device pointer of a contiguous CUDA tensor (None for None)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return t.data_ptr()


def dbl_array(values):
    vals = [float(v) for v in values]
    arr = (ctypes.c_double * max(1, len(vals)))(*vals)
    return arr


def device_status() -> int:
    """Synchronise the current stream and return (and clear) the device status word."""
    st = _c_int(0)
    call("dlx_device_status", stream_ptr(), ctypes.byref(st))
    return st.value
