"""Radix-2 line-FFT form of the padded centred FFT (pad * N a power of two) against the
FP64 oracle, against the DFT-GEMM form, and its adjoint. Tolerance: relative L2 <= 1e-5
(FP32 butterflies, ~log2(P) ulps); adjoint identity <= 1e-5.
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def field(n, seed, batch=1):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n))) / n


@pytest.mark.parametrize("n,pad,inverse,fl", [(32, 2, False, None), (64, 4, True, None),
                                              (256, 2, False, 3.0), (512, 2, False, None),
                                              (1024, 2, True, None)])
def test_radix_fft_matches_oracle(cuda, n, pad, inverse, fl):
    from dlux_gb300 import kernels
    wls = [1.0e-6, 1.3e-6]
    E = field(n, n + pad, len(wls))
    plan = kernels.FFTPlan(wls, n, 0.1 / n, pad, fl, inverse, variant="radix")
    got = plan.forward(torch.as_tensor(E, dtype=torch.complex64, device="cuda")).cpu().numpy()
    errs = []
    for b, wl in enumerate(wls):
        ref, _ = O.fft_prop(E[b], wl, 0.1 / n, fl, pad, inverse)
        errs.append(rel(got[b], ref))
    print(f"radix FFT n={n} pad={pad}: rel L2 {max(errs):.2e}")
    assert max(errs) < 1e-5


@pytest.mark.parametrize("center_in,center_out,fl", [(0.01, 0.0, 2.0), (0.0, 1e-6, None)])
def test_radix_fft_with_ramps_matches_gemm_form(cuda, center_in, center_out, fl):
    from dlux_gb300 import kernels
    n, pad = 64, 4
    E = field(n, 9)
    x = torch.as_tensor(E, dtype=torch.complex64, device="cuda")
    args = ([1e-6], n, 1 / 64, pad, fl, False, (center_in, center_out))
    a = kernels.FFTPlan(*args, variant="radix").forward(x).cpu().numpy()
    b = kernels.FFTPlan(*args, variant="fp32").forward(x).cpu().numpy()
    ref, _, _ = O.propagate_fft(E[0], 1e-6, 1 / 64, center_in, pad, fl, center_out)
    print(f"radix vs fp32 DFT-GEMM {rel(a, b):.2e}, radix vs oracle {rel(a[0], ref):.2e}")
    assert rel(a[0], ref) < 1e-5 and rel(a, b) < 1e-5


@pytest.mark.parametrize("n,pad", [(64, 2), (256, 4)])
def test_radix_fft_adjoint_identity(cuda, n, pad):
    from dlux_gb300 import kernels
    plan = kernels.FFTPlan([1e-6], n, 1 / n, pad, None, False, (0.003, 2e-7), variant="radix")
    P = n * pad
    x = torch.as_tensor(field(n, 1), dtype=torch.complex64, device="cuda")
    y = torch.as_tensor(field(P, 2), dtype=torch.complex64, device="cuda")
    lhs = torch.vdot(plan.forward(x).reshape(-1), y.reshape(-1)).item()
    rhs = torch.vdot(x.reshape(-1), plan.adjoint(y).reshape(-1)).item()
    err = abs(lhs - rhs) / abs(lhs)
    print(f"radix adjoint n={n} pad={pad}: {err:.2e}")
    assert err < 1e-5


def test_public_fft_selects_radix_for_large_pads(cuda):
    import dlux_gb300.utils as dlu
    from dlux_gb300 import kernels
    assert kernels.resolve_fft_variant(2048, 2) == 2
    assert kernels.resolve_fft_variant(512, 2) != 2      # the tensor-core GEMM form is faster
    assert kernels.resolve_fft_variant(2000, 2) != 2     # not a power of two
    E = field(2048, 4)[0]
    got, ps = dlu.FFT(torch.as_tensor(E, dtype=torch.complex64, device="cuda"), 1e-6, 1 / 2048,
                      None, 2, False)
    ref, ps_ref = O.fft_prop(E, 1e-6, 1 / 2048, None, 2, False)
    assert rel(got.cpu().numpy(), ref) < 1e-5
    with pytest.raises(ValueError):
        kernels.FFTPlan([1e-6], 500, 1 / 500, 2, variant="radix")
