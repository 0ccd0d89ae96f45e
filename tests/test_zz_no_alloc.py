"""The allocation-free MFT entry point, through the C ABI.

dlx_mft_forward_noalloc serves callers that may not allocate device memory
(for instance an XLA custom call running while XLA holds most of the GPU in
its own pool). It keeps its DFT matrices and intermediate field in a fixed
device array inside the library instead of in a plan. These tests call it
twice in a row -- different sizes, wavelengths and shifts, so the second call
runs on scratch that still holds the first call's contents -- and compare each
result with the plan-based dlx_mft_forward (FP32 form) and with the FP64
oracle, within the FP32 tolerance of the other MFT tests (relative L2 <= 2e-5).
They also check that device memory in use does not change across calls after
the first (which may load the library's device module), that sizes beyond the
fixed scratch are refused, and that a negative focal length is refused rather
than treated as the angular form.
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu

CASES = [
    # n_in, n_out, batch, ps_in, ps_out, focal, shift, inverse, wavelengths
    (256, 128, 2, 1 / 256, 9.7e-8, None, (0.0, 0.0), False, [1.0e-6, 1.2e-6]),
    (512, 512, 1, 1 / 512, 2.4e-8, 2.0, (1.5, -0.5), True, [0.8e-6]),
]


def _rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _noalloc(field, wls, n_out, ps_in, ps_out, focal=None, shift=(0.0, 0.0), inverse=False,
             out=None):
    import dlux_gb300._lib as L
    b, n_in = field.shape[0], field.shape[-1]
    if out is None:
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


def _oracle(E, wls, n_out, ps_in, ps_out, focal, shift, inverse):
    return np.stack([O.mft(E[i], wl, ps_in, n_out, ps_out, focal, shift, True, inverse)
                     for i, wl in enumerate(wls)])


def _fields(rng, b, n):
    E = (rng.normal(size=(b, n, n)) + 1j * rng.normal(size=(b, n, n))) / n
    return E, torch.as_tensor(E, dtype=torch.complex64, device="cuda")


def test_noalloc_matches_planned_mft_and_oracle_twice(cuda):
    rng = np.random.default_rng(2026)
    for n_in, n_out, b, ps_in, ps_out, fl, sh, inv, wls in CASES:
        E, field = _fields(rng, b, n_in)
        got = _noalloc(field, wls, n_out, ps_in, ps_out, fl, sh, inv)
        ref = _planned(field, wls, n_out, ps_in, ps_out, fl, sh, inv)
        assert got.shape == (b, n_out, n_out)
        got_np = got.cpu().numpy()
        assert _rel(got_np, ref.cpu().numpy()) < 2e-5
        assert _rel(got_np, _oracle(E, wls, n_out, ps_in, ps_out, fl, sh, inv)) < 2e-5


def test_noalloc_allocates_nothing_after_its_first_call(cuda):
    rng = np.random.default_rng(7)
    prepared = []
    for n_in, n_out, b, ps_in, ps_out, fl, sh, inv, wls in CASES:
        E, field = _fields(rng, b, n_in)
        out = torch.empty((b, n_out, n_out), dtype=torch.complex64, device="cuda")
        prepared.append((E, field, out, (wls, n_out, ps_in, ps_out, fl, sh, inv)))
    # set-up call: looks up the scratch array on this device
    E, field, out, a = prepared[0]
    _noalloc(field, *a, out=out)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    for E, field, out, a in prepared + prepared:
        _noalloc(field, *a, out=out)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert torch.cuda.memory_allocated() == alloc0
    assert free1 == free0
    for E, field, out, a in prepared:
        wls, n_out, ps_in, ps_out, fl, sh, inv = a
        assert _rel(out.cpu().numpy(), _oracle(E, wls, n_out, ps_in, ps_out, fl, sh, inv)) < 2e-5


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    field = torch.zeros((1, 1024, 1024), dtype=torch.complex64, device="cuda")
    with pytest.raises(ValueError, match="scratch"):
        _noalloc(field, [1e-6], 1024, 1 / 1024, 1e-8)
    # 592 x 592 needs 3 * 2803712 + 256 bytes, just over 8 MiB
    field = torch.zeros((1, 592, 592), dtype=torch.complex64, device="cuda")
    with pytest.raises(ValueError, match="scratch"):
        _noalloc(field, [1e-6], 592, 1 / 592, 1e-8)


def test_noalloc_rejects_negative_focal_length(cuda):
    field = torch.zeros((1, 64, 64), dtype=torch.complex64, device="cuda")
    with pytest.raises(ValueError, match="focal_length"):
        _noalloc(field, [1e-6], 32, 1 / 64, 1e-6, focal=-2.0)
