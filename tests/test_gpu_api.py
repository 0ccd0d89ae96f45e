"""The dLux-compatible API end to end on the GPU, against the FP64 oracle."""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def config1(seed=1):
    """Config 1: 256^2 pupil, 10% obscuration, Noll 4..13 ~ N(0, 50 nm), 1 um, 128^2 at 0.02"."""
    rng = np.random.default_rng(seed)
    T, B = O.circular_aperture(256, 1.0, oversample=5, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 14)))
    c = rng.normal(0, 50e-9, 10)
    R = rng.normal(size=(128, 128)).astype(np.float32)
    return T, B, c, R


def build_system(T, B, c, psf_npixels=128, pixel_scale=0.02, oversample=1):
    import dlux_gb300 as dl
    layers = [dl.TransmissiveLayer(torch.as_tensor(T, dtype=torch.float32, device="cuda"),
                                   normalise=True),
              dl.BasisLayer(torch.as_tensor(B, dtype=torch.float32, device="cuda"),
                            torch.as_tensor(c, dtype=torch.float32, device="cuda"))]
    return dl.AngularOpticalSystem(T.shape[-1], 1.0, layers, psf_npixels, pixel_scale, oversample)


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_config1_psf_and_gradient(cuda, variant):
    import dlux_gb300 as dl
    dl.set_variant(variant)
    try:
        T, B, c, R = config1()
        optics = build_system(T, B, c)
        coeffs = torch.as_tensor(c, dtype=torch.float32, device="cuda").requires_grad_(True)
        optics = optics.set("layers.BasisLayer.coefficients", coeffs)
        psf = optics.propagate(1e-6)
        opd = O.eval_basis(B, c)
        ref = O.poly_psf(T, opd, [1e-6], [1.0], 1.0, 128, float(O.arcsec2rad(0.02)))
        assert rel(psf.detach().cpu().numpy(), ref) < 1e-5
        loss = (psf * torch.as_tensor(R, device="cuda")).sum()
        loss.backward()
        Teff = T / np.sqrt((T ** 2).sum())
        g = O.poly_psf_grad(Teff, opd, [1e-6], [1.0], 1.0, 128, float(O.arcsec2rad(0.02)), R)
        gc_ref = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))
        err = rel(coeffs.grad.cpu().numpy(), gc_ref)
        print(f"config 1 {variant}: d loss / d c rel L2 {err:.2e}")
        assert err < 1e-5
    finally:
        dl.set_variant(None)


def test_transmission_gradient_through_normalise(cuda):
    import dlux_gb300 as dl
    T, B, c, R = config1(3)
    T = T * (1 + 0.01 * np.random.default_rng(4).normal(size=T.shape))
    optics = build_system(T, B, c, psf_npixels=64, pixel_scale=0.04)
    Tt = torch.as_tensor(T, dtype=torch.float32, device="cuda").requires_grad_(True)
    optics = optics.set("layers.TransmissiveLayer.transmission", Tt)
    psf = optics.propagate([0.9e-6, 1.1e-6], weights=[0.4, 0.6])
    G = np.random.default_rng(5).normal(size=(64, 64))
    (psf * torch.as_tensor(G, dtype=torch.float32, device="cuda")).sum().backward()
    # chain of a = T / sqrt(sum T^2) in FP64
    opd = O.eval_basis(B, c)
    S = (T ** 2).sum()
    Teff = T / np.sqrt(S)
    g = O.poly_psf_grad(Teff, opd, [0.9e-6, 1.1e-6], [0.4, 0.6], 1.0, 64,
                        float(O.arcsec2rad(0.04)), G)
    ge = g["g_amp"]
    gT = ge / np.sqrt(S) - T * (T * ge).sum() / S ** 1.5
    e = rel(Tt.grad.cpu().numpy(), gT)
    print(f"transmission gradient through the normalisation: {e:.2e}")
    assert e < 1e-5


def test_normalisation_beside_the_opd_matches_serial(cuda):
    """A fused pupil with a normalising transmission computes the normalisation on a
    side stream while the OPD is evaluated; the scale is the serial kernel's bits, and
    the PSF equals the one computed with the scale taken on the current stream."""
    from dlux_gb300 import autograd, kernels
    T, B, c, _ = config1(6)
    optics = build_system(T, B, c, psf_npixels=64, pixel_scale=0.04)
    amp, flag, opd, phase, tilt, scale = optics.fused_pupil()
    assert flag and scale is not None
    serial = kernels.amp_norm(amp)
    torch.cuda.synchronize()
    assert torch.equal(scale, serial)
    plan = optics.fused_plan([1e-6])
    w = torch.ones(1, device="cuda")
    a = autograd.poly_psf(plan, amp, opd, phase, w, True, tilt, scale)
    b = autograd.poly_psf(plan, amp, opd, phase, w, True, tilt)
    assert torch.equal(a, b)


def test_telescope_with_detector(cuda):
    import dlux_gb300 as dl
    T, B, c, R = config1(6)
    optics = build_system(T, B, c, psf_npixels=64, pixel_scale=0.02, oversample=4)
    flat = (1 + 0.02 * np.random.default_rng(7).normal(size=(64, 64))).astype(np.float32)
    det = dl.LayeredDetector([dl.Downsample(4), dl.ApplyPixelResponse(flat)])
    wls = np.linspace(0.8e-6, 1.2e-6, 5)
    src = dl.PointSource(wls, weights=np.arange(1, 6, dtype=float))
    tel = dl.Telescope(optics, src, det)
    img = tel.model().cpu().numpy()
    w = np.arange(1, 6) / 15.0
    psf = O.poly_psf(T, O.eval_basis(B, c), wls, w, 1.0, 256, float(O.arcsec2rad(0.005)))
    ref = O.downsample(psf, 4, mean=False) * flat
    assert img.shape == (64, 64)
    assert rel(img, ref) < 1e-5


def test_generic_layer_path_matches_fused(cuda):
    """A LayeredOpticalSystem with an explicit MFT layer runs layer by layer."""
    import dlux_gb300 as dl
    T, B, c, R = config1(8)
    Td = torch.as_tensor(T, dtype=torch.float32, device="cuda")
    Bd = torch.as_tensor(B, dtype=torch.float32, device="cuda")
    cd = torch.as_tensor(c, dtype=torch.float32, device="cuda")
    ps = float(O.arcsec2rad(0.02))
    layered = dl.LayeredOpticalSystem(256, 1.0, [dl.TransmissiveLayer(Td, normalise=True),
                                                 dl.BasisLayer(Bd, cd), dl.MFT(128, ps)])
    fused = dl.AngularOpticalSystem(256, 1.0, [dl.TransmissiveLayer(Td, normalise=True),
                                               dl.BasisLayer(Bd, cd)], 128, 0.02)
    wls = [0.9e-6, 1.0e-6]
    a = layered.propagate(wls).cpu().numpy()
    b = fused.propagate(wls).cpu().numpy()
    ref = O.poly_psf(T, O.eval_basis(B, c), wls, [0.5, 0.5], 1.0, 128, ps)
    assert rel(a, ref) < 1e-5
    assert rel(b, ref) < 1e-5


def test_source_offset_is_a_tilt(cuda):
    import dlux_gb300 as dl
    T, B, c, R = config1(9)
    optics = build_system(T, B, c, psf_npixels=64, pixel_scale=0.02)
    off = np.array([0.1, -0.05]) * np.pi / 180 / 3600
    psf = optics.propagate([1e-6], offset=off).cpu().numpy()
    ref = O.poly_psf(T, O.eval_basis(B, c), [1e-6], [1.0], 1.0, 64, float(O.arcsec2rad(0.02)),
                     offset=off)
    assert rel(psf, ref) < 1e-5


def test_point_sources_position_gradient(cuda):
    import dlux_gb300 as dl
    T, B, c, R = config1(10)
    optics = build_system(T, B, c, psf_npixels=32, pixel_scale=0.04)
    pos = torch.tensor([[0.05, 0.0], [-0.1, 0.07]], dtype=torch.float64) * (np.pi / 180 / 3600)
    pos.requires_grad_(True)
    src = dl.PointSources([1e-6], position=pos, flux=[1.0, 2.0])
    psf = src.model(optics)
    G = torch.as_tensor(np.random.default_rng(11).normal(size=(32, 32)), dtype=torch.float32,
                        device="cuda")
    (psf * G).sum().backward()
    assert pos.grad is not None and torch.isfinite(pos.grad).all()
    # central differences in FP64 on the oracle
    opd = O.eval_basis(B, c)
    Gn = G.cpu().numpy()

    def loss(p):
        tot = 0
        for (x, y), f in zip(p, [1.0, 2.0]):
            tot = tot + (Gn * O.poly_psf(T, opd, [1e-6], [f], 1.0, 32, float(O.arcsec2rad(0.04)),
                                         offset=(x, y))).sum()
        return tot
    p0 = pos.detach().numpy()
    # fourth-order central differences in FP64 (step 2e-9 rad: truncation ~1e-9)
    h = 2e-9
    fd = np.zeros_like(p0)
    for i in range(2):
        for j in range(2):
            d = np.zeros_like(p0)
            d[i, j] = h
            fd[i, j] = (-loss(p0 + 2 * d) + 8 * loss(p0 + d) - 8 * loss(p0 - d)
                        + loss(p0 - 2 * d)) / (12 * h)
    assert rel(pos.grad.numpy(), fd) < 1e-5


def test_reference_error_paths():
    """Shape errors of OpticalSystem.propagate raise ValueError (test_optical_systems.py:36-51)."""
    import dlux_gb300 as dl
    T, B, c, R = config1(12)
    optics = build_system(T[:64:4, :64:4], B[:, :64:4, :64:4], c, psf_npixels=16)
    with pytest.raises(ValueError):
        optics.propagate([1e-6, 2e-6], weights=[1.0])
    with pytest.raises(ValueError):
        optics.propagate([1e-6], offset=[0.0])
    with pytest.raises(ValueError):
        optics.propagate([1e-6], return_wf=True, return_psf=True)
