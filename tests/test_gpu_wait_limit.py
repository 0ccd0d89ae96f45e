"""Bounded waits of the tensor-core GEMM: an expired wait is reported, not hung.

Every mbarrier wait in the tensor-core GEMM has a wall-clock limit
(dlx_set_wait_limit_ns; 2 s by default). The test makes the waits run out
without faulting anything: the copy warp is told to issue no copies
(dlx_test_gemm_withhold_copies), so the MMA and epilogue warps wait on
barriers that nothing will complete, with no copy in flight. With the limit
at 1 ms each GEMM then records DLX_ERR_TIMEOUT in the device status word,
frees its tensor memory and returns. The test checks that status, that
reading it clears it, and that the next normal call on the same plan matches
the FP64 oracle (relative L2 <= 1e-5, the split-BF16 MFT tolerance).
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_expired_gemm_wait_reports_timeout_and_plan_recovers(cuda):
    import dlux_gb300 as dl
    import dlux_gb300._lib as L
    from dlux_gb300 import kernels
    if not dl.tensor_core_available():
        pytest.skip("tensor-core form unavailable on this device")
    wl, n_in, n_out, ps_in = 1.0e-6, 256, 128, 1 / 256
    ps_out = float(O.arcsec2rad(0.02))
    rng = np.random.default_rng(11)
    E = (rng.normal(size=(1, n_in, n_in)) + 1j * rng.normal(size=(1, n_in, n_in))) / n_in
    field = torch.as_tensor(E, dtype=torch.complex64, device="cuda")
    plan = kernels.MFTPlan([wl], n_in, ps_in, n_out, ps_out, variant="split_bf16")
    try:
        assert L.device_status() == L.DLX_OK  # nothing pending
        L.call("dlx_set_wait_limit_ns", 1_000_000)
        L.call("dlx_test_gemm_withhold_copies", 1)
        try:
            plan.forward(field)
            status = L.device_status()
        finally:
            L.call("dlx_test_gemm_withhold_copies", 0)
            L.call("dlx_set_wait_limit_ns", 0)
        assert status == L.DLX_ERR_TIMEOUT
        assert L.device_status() == L.DLX_OK  # reading the word cleared it
        out = plan.forward(field)
        assert L.device_status() == L.DLX_OK
        ref = O.mft(E[0], wl, ps_in, n_out, ps_out)
        assert _rel(out[0].cpu().numpy(), ref) < 1e-5
    finally:
        plan.close()
