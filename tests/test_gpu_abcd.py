"""ABCD propagators on the GPU against the oracle's FP64 restatements.

- The LCT runs as a chirped two-GEMM transform (XformPlan), in both forms.
  It is compared with the direct Collins sum for Fraunhofer, Fresnel and
  lens + free-space systems (including B < 0).
- The ASM runs as DFT, transfer function and inverse DFT (ASMPlan), and is
  compared with the oracle's NumPy-FFT ASM.
- Adjoint identities cover the reverse passes, and the layer calls of dLux's
  tests/layers/test_abcd_propagators.py are restated.

Tolerances are relative L2 errors: 1e-6 for the FP32 form, 1e-5 for the
split-BF16 form, as for the MFT.
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-6, "split_bf16": 1e-5}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def field(n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))


def c64(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.complex64, device="cuda")


SYSTEMS = {
    "fraunhofer": lambda: O.abcd_fraunhofer(2.0),
    "fresnel": lambda: O.abcd_free_space(0.2),
    "lens_then_space": lambda: O.compose_abcd([O.abcd_lens(1.5), O.abcd_free_space(0.4)]),
    "negative_B": lambda: O.compose_abcd([O.abcd_free_space(-0.3), O.abcd_mirror(2.0)]),
}


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
@pytest.mark.parametrize("system", list(SYSTEMS))
def test_lct_matches_collins_sum(cuda, variant, system):
    from dlux_gb300 import kernels
    from dlux_gb300.layers import abcd_propagators as ap
    M = SYSTEMS[system]()
    n, m = 64, 48
    wls = [0.9e-6, 1.1e-6]
    dx = 4e-5
    # output sampling: the Fraunhofer focal-plane scale, or the input scale
    B = float(M[0, 1])
    d_out = wls[0] * abs(B) / (n * dx) if system == "fraunhofer" else dx
    u = [field(n, 10 + k) for k in range(len(wls))]
    axes = ap.lct_axes(torch.as_tensor(M), wls, n, dx, 1e-5, m, d_out, -2e-5)
    plan = kernels.XformPlan(axes, axes, n, m, variant=variant)
    out = plan.forward(c64(np.stack(u))).cpu().numpy()
    for k, w in enumerate(wls):
        ref = O.lct_direct(u[k], O.coord_xs(n, dx, 1e-5), O.coord_xs(m, d_out, -2e-5), w, M)
        assert rel(out[k], ref) < TOL[variant], (k, rel(out[k], ref))


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_xform_and_asm_adjoint_identities(cuda, variant):
    from dlux_gb300 import kernels
    from dlux_gb300.layers import abcd_propagators as ap
    M = torch.as_tensor(O.compose_abcd([O.abcd_lens(1.5), O.abcd_free_space(0.4)]))
    n, m = 32, 40
    wls = [1e-6]
    axes = ap.lct_axes(M, wls, n, 3e-5, 0.0, m, 2e-5, 0.0)
    plans = [(kernels.XformPlan(axes, axes, n, m, variant=variant), m),
             (kernels.ASMPlan(wls, n, 48, 2e-5, 0.05, variant=variant), 48)]
    for plan, no in plans:
        x = c64(field(n, 1)[None])
        y = c64(field(no, 2)[None])
        ax = plan.forward(x)
        aty = plan.adjoint(y)
        lhs = torch.vdot(ax.flatten().to(torch.complex128), y.flatten().to(torch.complex128))
        rhs = torch.vdot(x.flatten().to(torch.complex128), aty.flatten().to(torch.complex128))
        # relative to the Cauchy-Schwarz bound: <Ax, y> of random vectors cancels
        scale = torch.linalg.vector_norm(ax) * torch.linalg.vector_norm(y)
        assert abs(lhs - rhs) / scale < TOL[variant]


@pytest.mark.parametrize("n,n_pad,dx,z,variant", [(16, 20, 1 / 16, 1.0, "fp32"),
                                                  (64, 128, 2e-5, 0.05, "split_bf16"),
                                                  (64, 128, 2e-5, 0.05, "fp32"),
                                                  (32, 64, 5e-7, 2e-6, "fp32")])
def test_asm_matches_oracle(cuda, n, n_pad, dx, z, variant):
    """Last case: dx near lambda, so the grid holds evanescent components."""
    from dlux_gb300 import kernels
    wls = [0.8e-6, 1.2e-6]
    u = [field(n, 20 + k) for k in range(len(wls))]
    plan = kernels.ASMPlan(wls, n, n_pad, dx, z, variant=variant)
    out = plan.forward(c64(np.stack(u))).cpu().numpy()
    for k, w in enumerate(wls):
        ref = O.asm_prop(u[k], dx, w, z, n_pad)
        assert rel(out[k], ref) < TOL[variant], (k, rel(out[k], ref))


def test_layer_calls_of_the_reference_tests(cuda):
    import dlux_gb300 as dl
    from dlux_gb300.coordinates import CoordSpec, PadSpec
    from dlux_gb300.layers import abcd_propagators as ap

    wf = dl.Wavefront(npixels=16, diameter=1.0, wavelength=1e-6)
    out = ap.MFTPropagator([ap.ABCDFreeSpace(1.0)], CoordSpec(n=8, d=1 / 32, c=0.0))(wf)
    assert isinstance(out, dl.Wavefront) and out.npixels == 8
    assert np.allclose(out.pixel_scale, 1 / 32)
    for prop, n_out in [
            (ap.FFTPropagator([ap.ABCDConjugatePlane(1.0)], CoordSpec(n=20, c=0.0)), 20),
            (ap.FFTPropagator([ap.ABCDConjugatePlane(1.0)], PadSpec(pad=2, crop=2, c=0.0)), 16),
            (ap.ASMPropagator(1.0, CoordSpec(n=20, c=None)), 20),
            (ap.ASMPropagator(1.0, PadSpec(pad=2, crop=2, c=0.0)), 16)]:
        out = prop(wf)
        assert isinstance(out, dl.Wavefront) and out.npixels == n_out
        assert torch.isfinite(out.phasor.real).all() and torch.isfinite(out.phasor.imag).all()


def test_fft_propagator_is_the_lct_on_the_fft_grid(cuda):
    """FFTPropagator with the Fraunhofer system: the focal-plane field on the
    FFT grid, i.e. -i dx / d_fft times dLux's MFT to that grid, and the
    padded-crop variant is its centre."""
    import dlux_gb300 as dl
    from dlux_gb300.coordinates import PadSpec
    from dlux_gb300.layers import abcd_propagators as ap
    n, f, wl = 32, 3.0, 1e-6
    u = field(n, 5)
    wf = dl.Wavefront.from_phasor(c64(u), wl, diameter=1.0)
    prop = ap.FFTPropagator([ap.ABCDConjugatePlane(f)], PadSpec(pad=2, crop=1, c=0.0))
    out = prop(wf)
    P, dx = 2 * n, 1.0 / n
    d_fft = wl * f / (P * dx)
    assert np.isclose(out.pixel_scale, d_fft)
    ref = (-1j * dx / d_fft) * O.mft(u, wl, dx, P, d_fft, focal_length=f)
    assert rel(out.phasor.cpu().numpy(), ref) < 1e-5
    cropped = ap.FFTPropagator([ap.ABCDConjugatePlane(f)], PadSpec(pad=2, crop=2, c=0.0))(wf)
    np.testing.assert_allclose(cropped.phasor.cpu().numpy(),
                               out.phasor.cpu().numpy()[n // 2:n // 2 + n, n // 2:n // 2 + n],
                               rtol=0, atol=1e-6 * np.abs(ref).max())


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_gradient_through_the_propagators(cuda, variant):
    """Reverse pass through MFTPropagator and ASMPropagator (the plans'
    adjoints) against central differences of the FP64 oracle, for the
    derivative of sum |out|^2 R along a random phase direction: |d - d_ref| <=
    tol (|d_ref| + ||g * v||_2), i.e. relative to the size of the sum's terms.
    tol is 1e-5, and 3e-5 for the split-BF16 form on this 32-pixel grid, where
    a transform sums too few terms (K = 32) for the operand splits' rounding to
    average out (the same bound as the MFT fixtures at K = 32)."""
    import dlux_gb300 as dl
    dl.set_variant(variant)
    try:
        _gradient_through_the_propagators(1e-5 if variant == "fp32" else 3e-5)
    finally:
        dl.set_variant(None)


def _gradient_through_the_propagators(tol):
    import dlux_gb300 as dl
    from dlux_gb300.coordinates import CoordSpec, PadSpec
    from dlux_gb300.layers import abcd_propagators as ap
    n, wl = 32, 1e-6
    rng = np.random.default_rng(7)
    amp = np.abs(field(n, 3))
    phi0 = rng.normal(size=(n, n))
    dphi = rng.normal(size=(n, n))
    Mf = O.abcd_fraunhofer(2.0)
    # ASM in the Fresnel regime (dx^2 N / (lambda z) < 1), where the phase
    # direction changes sum |out|^2 R by a few per cent of its scale
    dx_f, dx_a = 1.0 / n, 20e-6
    cases = [
        (ap.MFTPropagator([ap.ABCDConjugatePlane(2.0)], CoordSpec(n=24, d=4e-6, c=0.0)),
         lambda u: O.lct_direct(u, O.coord_xs(n, dx_f), O.coord_xs(24, 4e-6), wl, Mf), 24,
         dx_f),
        (ap.ASMPropagator(0.02, PadSpec(pad=2, crop=1)),
         lambda u: O.asm_prop(u, dx_a, wl, 0.02, 2 * n), 2 * n, dx_a),
    ]
    for prop, ref_fn, m, dx in cases:
        R = rng.normal(size=(m, m))
        ph = torch.as_tensor(phi0, dtype=torch.float32, device="cuda").requires_grad_(True)
        ampt = torch.as_tensor(amp, dtype=torch.float32, device="cuda")
        u = torch.complex(ampt * torch.cos(ph), ampt * torch.sin(ph))
        wf = dl.Wavefront.from_phasor(u, wl, diameter=n * dx)
        out = prop(wf).phasor
        loss = ((out.real ** 2 + out.imag ** 2) * torch.as_tensor(R, dtype=torch.float32,
                                                                  device="cuda")).sum()
        loss.backward()

        def f(e):
            v = ref_fn(amp * np.exp(1j * (phi0 + e * dphi)))
            return float((np.abs(v) ** 2 * R).sum())
        # fourth-order central difference in FP64 (truncation ~h^4 = 1e-12); the
        # derivative d = sum_p g_p v_p is compared relative to its terms' size
        h = 1e-3
        fd = (-f(2 * h) + 8 * f(h) - 8 * f(-h) + f(-2 * h)) / (12 * h)
        terms = ph.grad.double().cpu().numpy() * dphi
        d = float(terms.sum())
        scale = abs(fd) + float(np.linalg.norm(terms))
        print(f"{type(prop).__name__}: derivative {d:.6e} vs {fd:.6e}, "
              f"{abs(d - fd) / scale:.2e} of scale")
        assert abs(d - fd) <= tol * scale, (d, fd)
