"""The allocation-free MFT entry point, through the C ABI.

dlx_mft_forward_noalloc serves callers that may not allocate device memory
(for instance an XLA custom call running while XLA holds most of the GPU in
its own pool). It keeps its DFT matrices and intermediate field in a fixed
device array inside the library instead of in a plan. These tests call it
twice in a row -- different sizes, wavelengths and shifts, so the second call
runs on scratch that still holds the first call's contents -- and compare each
result with the plan-based dlx_mft_forward (FP32 form) within the FP32
tolerance of the other MFT tests (relative L2 <= 2e-5), and check that sizes
beyond the fixed scratch are refused.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.cpu().numpy().astype(np.complex128)
    b = b.cpu().numpy().astype(np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _noalloc(field, wls, n_out, ps_in, ps_out, focal=None, shift=(0.0, 0.0), inverse=False):
    import dlux_gb300._lib as L
    b, n_in = field.shape[0], field.shape[-1]
    out = torch.empty((b, n_out, n_out), dtype=torch.complex64, device="cuda")
    L.call("dlx_mft_forward_noalloc", L.ptr(field), b, n_in, float(ps_in), n_out, float(ps_out),
           L.dbl_array(wls), 0.0 if focal is None else float(focal), float(shift[0]),
           float(shift[1]), int(inverse), L.ptr(out), L.stream_ptr())
    return out


def _planned(field, wls, n_out, ps_in, ps_out, focal=None, shift=(0.0, 0.0), inverse=False):
    from dlux_gb300 import kernels
    plan = kernels.MFTPlan(wls, field.shape[-1], ps_in, n_out, ps_out, focal, shift, inverse,
                           variant="fp32")
    try:
        out = plan.forward(field)
        torch.cuda.synchronize()
        return out
    finally:
        plan.close()


def test_noalloc_matches_planned_mft_twice(cuda):
    rng = np.random.default_rng(2026)
    cases = [
        # n_in, n_out, batch, ps_in, ps_out, focal, shift, inverse, wavelengths
        (256, 128, 2, 1 / 256, 9.7e-8, None, (0.0, 0.0), False, [1.0e-6, 1.2e-6]),
        (512, 512, 1, 1 / 512, 2.4e-8, 2.0, (1.5, -0.5), True, [0.8e-6]),
    ]
    for n_in, n_out, b, ps_in, ps_out, fl, sh, inv, wls in cases:
        E = (rng.normal(size=(b, n_in, n_in)) + 1j * rng.normal(size=(b, n_in, n_in))) / n_in
        field = torch.as_tensor(E, dtype=torch.complex64, device="cuda")
        got = _noalloc(field, wls, n_out, ps_in, ps_out, fl, sh, inv)
        ref = _planned(field, wls, n_out, ps_in, ps_out, fl, sh, inv)
        assert got.shape == (b, n_out, n_out)
        assert _rel(got, ref) < 2e-5


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    field = torch.zeros((1, 1024, 1024), dtype=torch.complex64, device="cuda")
    with pytest.raises(ValueError, match="scratch"):
        _noalloc(field, [1e-6], 1024, 1 / 1024, 1e-8)
