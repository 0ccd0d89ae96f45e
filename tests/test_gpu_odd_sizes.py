"""Sides that are not multiples of 8 on the tensor cores.

TMA wants 16-byte row pitches, so split-BF16 operands pad each row to a
multiple of 8 elements (split_ld); the tensor maps declare the true extent,
so the padding is never read. These tests run the split form on such sides
and compare it with the FP64 oracle: the MFT and its adjoint, the padded FFT
as a DFT-GEMM pair, and the fused polychromatic PSF with its gradient (both
DFT-operand modes), with sides that are odd (row pitches 8 + k), multiples of
4 (the four-pixel phasor path) and smaller than one 32-element K block.

Tolerances (relative L2), for transforms, PSFs and gradients alike: 1e-5 when
every side is at least 64, 3e-5 below that (too few terms in a sum for the
operand splits' rounding to average out, as in the other transform tests).
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


def field(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / n


def c64(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.complex64, device="cuda")


def f32(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device="cuda")


def test_automatic_choice_is_the_split_form_for_every_side(cuda):
    import dlux_gb300._lib as L
    from dlux_gb300 import kernels
    if not kernels.tensor_core_available():
        pytest.skip("tensor-core form unavailable on this device")
    for n, m in [(300, 100), (33, 17), (17, 33), (75, 45), (512, 512)]:
        assert kernels.resolve_variant(n, m) == L.VARIANT_SPLIT_BF16


@pytest.mark.parametrize("n_in,n_out", [(33, 17), (17, 33), (300, 100), (100, 300), (75, 150)])
def test_mft_and_adjoint_match_oracle(cuda, n_in, n_out):
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    dl.set_variant("split_bf16")
    try:
        wl, ps_in = 1e-6, 1.0 / n_in
        ps_out = float(O.arcsec2rad(0.013))
        shift = (0.3, -0.7)
        E = field(n_in, 2)
        x = c64(E).requires_grad_(True)
        out = dlu.MFT(x, wl, ps_in, n_out, ps_out, None, shift)
        ref = O.mft(E, wl, ps_in, n_out, ps_out, None, shift)
        tol = 1e-5 if min(n_in, n_out) >= 64 else 3e-5
        e_f = rel(out.detach().cpu().numpy(), ref)
        # adjoint: the gradient of Re<out, y> w.r.t. the input is MFT^H y
        y = field(n_out, 3)
        yt = c64(y)
        (out.real * yt.real + out.imag * yt.imag).sum().backward()
        xm = O.transfer_matrix(wl, n_in, ps_in, n_out, ps_out, shift[0])
        ym = O.transfer_matrix(wl, n_in, ps_in, n_out, ps_out, shift[1])
        s = O.calc_nfringes(wl, n_in, ps_in, n_out, ps_out) / (n_in * n_out)
        # forward F = s ym^T E xm (rows y, columns x); its adjoint
        g_ref = s * (ym.conj() @ y @ xm.conj().T)
        e_a = rel(x.grad.cpu().numpy(), g_ref)
        print(f"MFT {n_in} -> {n_out}: forward {e_f:.2e}, adjoint {e_a:.2e}")
        assert out.shape == (n_out, n_out)
        assert e_f < tol and e_a < tol
    finally:
        dl.set_variant(None)


@pytest.mark.parametrize("n,pad,inverse", [(45, 2, False), (100, 2, True), (36, 3, False)])
def test_fft_dft_gemm_matches_oracle(cuda, n, pad, inverse):
    from dlux_gb300 import kernels
    import dlux_gb300._lib as L
    E = field(n, 5)
    plan = kernels.FFTPlan([1e-6], n, 1.0 / n, pad, 2.0, inverse, None, "split_bf16")
    try:
        assert plan.variant == L.VARIANT_SPLIT_BF16
        got = plan.forward(c64(E)[None])[0].cpu().numpy()
    finally:
        plan.close()
    ref, _ = O.fft_prop(E, 1e-6, 1.0 / n, 2.0, pad, inverse)
    err = rel(got, ref)
    print(f"FFT {n} pad {pad}: {err:.2e}")
    assert got.shape == ref.shape
    assert err < (1e-5 if n >= 64 else 3e-5)


@pytest.mark.parametrize("operand_mode", [0, 1])
@pytest.mark.parametrize("n,m,L", [(300, 100, 4), (75, 45, 3), (74, 90, 2), (132, 260, 2)])
def test_poly_psf_and_gradient_match_oracle(cuda, operand_mode, n, m, L):
    from dlux_gb300 import kernels
    import dlux_gb300.utils as dlu
    rng = np.random.default_rng(n + m)
    # the package's aperture and basis builders (pinned to dLux's on even grids):
    # dLux's own basis is NaN at the centre pixel of an odd grid (0 ** negative
    # power times a zero coefficient), where the package takes the limit
    T, B = dlu.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                                 zernike_nolls=list(range(4, 14)))
    T = np.asarray(T.cpu() if hasattr(T, "cpu") else T, np.float64)
    B = np.asarray(B.cpu() if hasattr(B, "cpu") else B, np.float64)
    opd = O.eval_basis(B, rng.normal(0, 40e-9, 10))
    wls = np.linspace(0.8e-6, 1.2e-6, L)
    w = rng.dirichlet(np.ones(L))
    ps_out = float(O.arcsec2rad(0.02))
    G = rng.normal(size=(m, m))
    ref_psf = O.poly_psf(T, opd, wls, w, 1.0, m, ps_out)
    Teff = T / np.sqrt((T ** 2).sum())
    ref = O.poly_psf_grad(Teff, opd, wls, w, 1.0, m, ps_out, G)
    plan = kernels.PolyPlan(wls, n, 1.0 / n, m, ps_out, variant="split_bf16",
                            operand_mode=operand_mode)
    try:
        amp = f32(T)
        scale = kernels.amp_norm(amp)
        psf = plan.psf(amp, scale, f32(opd), None, f32(w)).cpu().numpy()
        gr = plan.grad(amp, scale, f32(opd), None, f32(w), f32(G))
        e_psf = rel(psf, ref_psf)
        e_opd = rel(gr["opd"].cpu().numpy(), ref["g_opd"])
        e_amp = rel(gr["amp"].cpu().numpy(), ref["g_amp"])
    finally:
        plan.close()
    print(f"poly {n} -> {m}, L={L}, operand mode {operand_mode}: PSF {e_psf:.2e}, "
          f"g_opd {e_opd:.2e}, g_amp {e_amp:.2e}")
    tol = 1e-5 if min(n, m) >= 64 else 3e-5
    assert e_psf < tol and e_opd < tol and e_amp < tol
