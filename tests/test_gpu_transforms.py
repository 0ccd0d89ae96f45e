"""GPU parity of the transfer matrix, MFT and FFT against the FP64 oracle.

Tolerances (relative L2 error against the FP64 restatement of dLux):
FP32 form <= 2e-5, split-BF16 tensor-core form <= 1e-5 on transforms whose
K dimension is at least 64 (smaller K is covered with a looser 3e-5).
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu

VARIANTS = ["fp32", "split_bf16"]


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def field(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / n


def test_transfer_matrix_matches_oracle(cuda):
    import dlux_gb300.utils as dlu
    for (wl, n_in, ps_in, n_out, ps_out, shift, fl, inv) in [
        (1.0, 32, 0.1, 16, 0.05, 1.0, 2.0, False),
        (1.0e-6, 256, 1 / 256, 128, O.arcsec2rad(0.02), 0.0, None, False),
        (0.8e-6, 33, 0.03, 17, 1e-7, -2.5, None, True),
    ]:
        got = dlu.transfer_matrix(wl, n_in, ps_in, n_out, ps_out, shift, fl, 0.0, inv)
        ref = O.transfer_matrix(wl, n_in, ps_in, n_out, ps_out, shift, fl, 0.0, inv)
        assert got.shape == (n_in, n_out)
        assert rel(got.cpu().numpy(), ref) < 1e-6


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("case", [
    # n_in, n_out, ps_in, ps_out, focal, shift, pixel, inverse, wl
    (32, 16, 0.1, 0.05, 2.0, (1.0, -2.0), True, False, 1.0),
    (32, 16, 0.1, 0.05, 2.0, (1.0, -2.0), False, True, 1.0),
    (32, 16, 0.1, 0.05, None, (0.0, 0.0), True, True, 1.0),
    (256, 128, 1 / 256, float(O.arcsec2rad(0.02)), None, (0.0, 0.0), True, False, 1e-6),
    (64, 96, 1 / 64, float(O.arcsec2rad(0.01)), None, (0.5, 3.0), True, False, 0.9e-6),
    (128, 512, 1 / 128, float(O.arcsec2rad(0.005)), None, (0.0, 0.0), True, False, 1.2e-6),
])
def test_mft_matches_oracle(cuda, variant, case):
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    n_in, n_out, ps_in, ps_out, fl, shift, pixel, inv, wl = case
    dl.set_variant(variant)
    try:
        E = field(n_in, 1)
        got = dlu.MFT(torch.as_tensor(E, dtype=torch.complex64, device="cuda"), wl, ps_in,
                      n_out, ps_out, fl, shift, pixel, inv)
        ref = O.mft(E, wl, ps_in, n_out, ps_out, fl, shift, pixel, inv)
        tol = 1e-5 if (variant == "split_bf16" and n_in >= 64) else 3e-5
        assert got.shape == (n_out, n_out)
        assert torch.isfinite(torch.view_as_real(got)).all()
        assert rel(got.cpu().numpy(), ref) < tol
    finally:
        dl.set_variant(None)


@pytest.mark.parametrize("variant", VARIANTS)
def test_mft_odd_sizes(cuda, variant):
    """Odd sides in both forms (the split form pads its operand rows to 8)."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    dl.set_variant(variant)
    try:
        E = field(33, 2)
        got = dlu.MFT(torch.as_tensor(E, dtype=torch.complex64, device="cuda"), 1e-6, 0.03, 17,
                      1e-7, None, (0.3, -0.7))
        ref = O.mft(E, 1e-6, 0.03, 17, 1e-7, None, (0.3, -0.7))
        assert rel(got.cpu().numpy(), ref) < 3e-5
    finally:
        dl.set_variant(None)


@pytest.mark.parametrize("variant", VARIANTS)
def test_mft_batched_wavelengths(cuda, variant):
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    dl.set_variant(variant)
    try:
        wls = [0.8e-6, 1.0e-6, 1.2e-6]
        E = np.stack([field(128, s) for s in range(3)])
        ps_out = float(O.arcsec2rad(0.01))
        got = dlu.MFT(torch.as_tensor(E, dtype=torch.complex64, device="cuda"), wls, 1 / 128,
                      64, ps_out).cpu().numpy()
        for i, wl in enumerate(wls):
            assert rel(got[i], O.mft(E[i], wl, 1 / 128, 64, ps_out)) < 3e-5
    finally:
        dl.set_variant(None)


@pytest.mark.parametrize("variant", VARIANTS)
def test_mft_shift_units_are_consistent(cuda, variant):
    """Reference test: pixel shift == physical shift scaled by the pixel scale."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    dl.set_variant(variant)
    try:
        ph = torch.ones((32, 32), dtype=torch.complex64, device="cuda")
        shift = np.array([1.0, -2.0])
        a = dlu.MFT(ph, 1.0, 0.1, 16, 0.05, 2.0, shift, pixel=True)
        b = dlu.MFT(ph, 1.0, 0.1, 16, 0.05, 2.0, shift * 0.05, pixel=False)
        assert torch.allclose(a, b, rtol=1e-6, atol=1e-6)
    finally:
        dl.set_variant(None)


@pytest.mark.parametrize("variant", VARIANTS)
def test_mft_adjoint_identity(cuda, variant):
    """<MFT x, y> == <x, MFT^H y> through torch autograd (the adjoint kernel)."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    dl.set_variant(variant)
    try:
        x = torch.as_tensor(field(128, 3), dtype=torch.complex64, device="cuda")
        y = torch.as_tensor(field(64, 4), dtype=torch.complex64, device="cuda")
        x.requires_grad_(True)
        out = dlu.MFT(x, 1e-6, 1 / 128, 64, float(O.arcsec2rad(0.01)))
        # real inner product Re<out, y>; its gradient w.r.t. x is MFT^H y
        (out.real * y.real + out.imag * y.imag).sum().backward()
        g = x.grad.cpu().numpy().astype(np.complex128)
        ay = O.transfer_matrix(1e-6, 128, 1 / 128, 64, float(O.arcsec2rad(0.01)))
        s = O.calc_nfringes(1e-6, 128, 1 / 128, 64, float(O.arcsec2rad(0.01))) / (128 * 64)
        ref = s * (ay.conj() @ y.cpu().numpy() @ ay.conj().T)
        assert rel(g, ref) < 3e-5
    finally:
        dl.set_variant(None)


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("pad,inverse,fl", [(2, False, 2.0), (2, True, 2.0), (1, False, None),
                                            (3, False, None)])
def test_fft_matches_oracle(cuda, variant, pad, inverse, fl):
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    dl.set_variant(variant)
    try:
        E = field(32, 5)
        got, ps = dlu.FFT(torch.as_tensor(E, dtype=torch.complex64, device="cuda"), 1.0, 0.1,
                          fl, pad, inverse)
        ref, ps_ref = O.fft_prop(E, 1.0, 0.1, fl, pad, inverse)
        assert got.shape == (32 * pad, 32 * pad)
        assert abs(ps - ps_ref) < 1e-12 * abs(ps_ref)
        assert rel(got.cpu().numpy(), ref) < 3e-5
    finally:
        dl.set_variant(None)


def test_fft_round_trip_no_padding(cuda):
    """Reference test: forward then inverse FFT recovers the input (rtol = atol = 1e-6)."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    dl.set_variant("fp32")
    try:
        ph = torch.ones((32, 32), dtype=torch.complex64, device="cuda")
        fwd, _ = dlu.FFT(ph, 1.0, 0.1, None, 1, False)
        back, _ = dlu.FFT(fwd, 1.0, 0.1, None, 1, True)
        assert torch.allclose(back, ph, rtol=1e-6, atol=1e-6)
    finally:
        dl.set_variant(None)


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("center_in,center_out,fl", [(0.0, 0.0, None), (0.01, 0.0, 2.0),
                                                     (0.0, 1e-6, None)])
def test_propagate_fft_with_ramps(cuda, variant, center_in, center_out, fl):
    import dlux_gb300 as dl
    dl.set_variant(variant)
    try:
        E = field(64, 6)
        wf = dl.Wavefront.from_phasor(E, 1e-6, pixel_scale=1 / 64, center=[center_in])
        out = wf.propagate_FFT(pad=2, focal_length=fl, spec_out=dl.CoordSpec(c=center_out))
        ref, ps, c = O.propagate_fft(E, 1e-6, 1 / 64, center_in, 2, fl, center_out)
        assert abs(out.pixel_scale - ps) < 1e-12 * ps and out.center == c
        assert rel(out.phasor.cpu().numpy(), ref) < 3e-5
    finally:
        dl.set_variant(None)
