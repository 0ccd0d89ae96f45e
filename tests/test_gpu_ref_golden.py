"""The CUDA path, through the public API, against outputs made by dLux itself.

tests/golden/ref_*.npz hold dLux v0.16.0's own outputs (its unmodified code
run in float64 by tests/golden/make_ref_golden.py); gradients are fourth-order
central differences of dLux's forward pass, accurate far below the tolerances
here. Inputs are rebuilt from tests/golden/ref_inputs.py.

Tolerances (relative L2 unless stated): transforms 1e-5 (3e-5 for the
split-BF16 form at K = 32, where an MFT sums too few terms for the operand
splits' rounding to average out); transfer matrices 1e-6; system images,
PSFs and gradient vectors 1e-5 in both arithmetic forms. A directional
derivative d = sum_i g_i v_i along a seeded direction v is checked as
|d - d_ref| <= 1e-5 (|d_ref| + ||g * v||_2), i.e. relative to the size of
the sum's own terms.
"""

import os
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)
import ref_inputs as RI  # noqa: E402

VARIANTS = ["split_bf16", "fp32"]
F32 = dict(dtype=torch.float32, device="cuda")


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def load(name):
    return np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))


def dd_ok(g, v, d_ref, tol=1e-5):
    g = np.asarray(g, np.float64)
    v = np.asarray(v, np.float64)
    d = float((g * v).sum())
    scale = abs(d_ref) + float(np.linalg.norm(g * v))
    print(f"  directional derivative {d:.6e} vs dLux {d_ref:.6e}: "
          f"{abs(d - d_ref) / scale:.2e} of scale")
    return abs(d - d_ref) <= tol * scale


@pytest.fixture
def variant(request):
    import dlux_gb300 as dl
    dl.set_variant(request.param)
    yield request.param
    dl.set_variant(None)


@pytest.mark.parametrize("variant", VARIANTS, indirect=True)
@pytest.mark.parametrize("case", RI.MFT_CASES, ids=[c[0] for c in RI.MFT_CASES])
def test_mft_matches_dlux(cuda, variant, case):
    import dlux_gb300.utils as dlu
    name, n_in, n_out, ps_in, ps_out, fl, shift, pixel, inv, wl = case
    ref = load("utils")
    E = torch.as_tensor(RI.case_field(name, n_in), dtype=torch.complex64, device="cuda")
    got = dlu.MFT(E, wl, ps_in, n_out, ps_out, focal_length=fl, shift=shift, pixel=pixel,
                  inverse=inv)
    err = rel(got.cpu().numpy(), ref[f"mft_{name}"])
    tol = 3e-5 if (variant == "split_bf16" and n_in <= 33) else 1e-5
    print(f"MFT {name} {variant}: {err:.2e}")
    assert err < tol
    if f"tm_{name}" in ref:
        tm = dlu.transfer_matrix(wl, n_in, ps_in, n_out, ps_out, shift[0], fl, 0.0, inv)
        assert rel(tm.cpu().numpy(), ref[f"tm_{name}"]) < 1e-6


@pytest.mark.parametrize("variant", VARIANTS, indirect=True)
@pytest.mark.parametrize("case", RI.FFT_CASES, ids=[c[0] for c in RI.FFT_CASES])
def test_fft_matches_dlux(cuda, variant, case):
    import dlux_gb300.utils as dlu
    name, n, ps, wl, fl, pad, inv = case
    ref = load("utils")
    E = torch.as_tensor(RI.case_field(name, n, salt=7), dtype=torch.complex64, device="cuda")
    got, ps_out = dlu.FFT(E, wl, ps, focal_length=fl, pad=pad, inverse=inv)
    err = rel(got.cpu().numpy(), ref[f"fft_{name}"])
    print(f"FFT {name} {variant}: {err:.2e}")
    tol = 3e-5 if (variant == "split_bf16" and n <= 33) else 1e-5
    assert err < tol
    assert abs(float(ps_out) - float(ref[f"fft_ps_{name}"])) <= 1e-12 * abs(float(ps_out))


@pytest.mark.parametrize("variant", VARIANTS, indirect=True)
def test_cfg1_psf_and_gradient_match_dlux(cuda, variant):
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    r, inp = load("cfg1"), RI.cfg1()
    T, B = dlu.circular_aperture(256, 1.0, oversample=1, secondary_diameter=0.1,
                                 zernike_nolls=inp["nolls"])
    c = torch.as_tensor(inp["coeffs"], **F32).requires_grad_(True)
    optics = dl.AngularOpticalSystem(256, 1.0, [dl.TransmissiveLayer(T, normalise=True),
                                                dl.BasisLayer(B, c)], 128, 0.02, 1)
    psf = optics.propagate(inp["wavelengths"])
    (psf * torch.as_tensor(inp["R"], **F32)).sum().backward()
    e_psf, e_g = rel(psf.detach().cpu().numpy(), r["psf"]), rel(c.grad.cpu().numpy(), r["grad"])
    print(f"cfg1 {variant}: PSF {e_psf:.2e}, gradient {e_g:.2e}")
    assert e_psf < 1e-5 and e_g < 1e-5


@pytest.mark.parametrize("variant", VARIANTS, indirect=True)
def test_unaligned_system_matches_dlux(cuda, variant):
    """100^2 pupil -> 67^2 PSF, 4 weighted wavelengths: sides that are not multiples of
    8, so the split form runs with padded operand rows."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    r, inp = load("unaligned"), RI.unaligned()
    T, B = dlu.circular_aperture(100, 1.0, oversample=1, secondary_diameter=0.1,
                                 zernike_nolls=inp["nolls"])
    c = torch.as_tensor(inp["coeffs"], **F32).requires_grad_(True)
    optics = dl.AngularOpticalSystem(100, 1.0, [dl.TransmissiveLayer(T, normalise=True),
                                                dl.BasisLayer(B, c)], 67, 0.03, 1)
    psf = optics.propagate(inp["wavelengths"], weights=torch.as_tensor(inp["weights"], **F32))
    (psf * torch.as_tensor(inp["R"], **F32)).sum().backward()
    e_psf, e_g = rel(psf.detach().cpu().numpy(), r["psf"]), rel(c.grad.cpu().numpy(), r["grad"])
    print(f"unaligned {variant}: PSF {e_psf:.2e}, gradient {e_g:.2e}")
    assert e_psf < 1e-5 and e_g < 1e-5


@pytest.mark.parametrize("variant", VARIANTS, indirect=True)
def test_cfg2_image_and_gradient_match_dlux(cuda, variant):
    """The benchmark workload at full size: 512^2 pupil, 64 wavelengths, 512^2 focal,
    4 x 4 downsample, all through the public API."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    r, inp = load("cfg2"), RI.cfg2()
    T, B = dlu.circular_aperture(512, 1.0, oversample=5, secondary_diameter=0.1,
                                 spider_width=0.01, spider_angles=(0, 90, 180, 270),
                                 zernike_nolls=inp["nolls"])
    c = torch.as_tensor(inp["coeffs"], **F32).requires_grad_(True)
    optics = dl.AngularOpticalSystem(512, 1.0, [dl.TransmissiveLayer(T, normalise=True),
                                                dl.BasisLayer(B, c)], 128, 0.02, 4)
    det = dl.LayeredDetector([dl.Downsample(4)])
    img = det.model(optics.propagate(inp["wavelengths"],
                                     weights=torch.as_tensor(inp["weights"], **F32),
                                     return_psf=True))
    (img * torch.as_tensor(inp["R"], **F32)).sum().backward()
    e_img, e_g = rel(img.detach().cpu().numpy(), r["image"]), rel(c.grad.cpu().numpy(), r["grad"])
    print(f"cfg2 {variant}: image {e_img:.2e}, gradient {e_g:.2e}")
    assert e_img < 1e-5 and e_g < 1e-5


@pytest.mark.parametrize("variant", VARIANTS, indirect=True)
def test_cfg3_phase_retrieval_matches_dlux(cuda, variant):
    """Config 3 at full size: image through the flat field, Poisson NLL, coefficient
    gradient, and directional derivatives w.r.t. amplitude and flat field.

    The NLL's cotangent 1 - d/m magnifies the image's relative error by up to
    ~sqrt(counts) (~1e2 here), so the reverse pass is checked on the reference's
    own cotangent: dL/dimage at the FP64 oracle's image (pinned to dLux's to 2e-16)
    is backpropagated through the device's reverse kernels, and the gradients must
    match dLux's within 1e-5. The end-to-end autograd gradient is held to 1e-4."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    from oracle import dlux_oracle as O
    r, inp = load("cfg3"), RI.cfg3()
    T, B = dlu.circular_aperture(512, 1.0, oversample=1, secondary_diameter=0.1,
                                 zernike_nolls=inp["nolls"])
    Tn = T.cpu().numpy().astype(np.float64)
    A0 = Tn * (1.0 + inp["amp_pert"])
    scale = float(r["scale"])
    data_np = r["data"].astype(np.float64)

    def run(cotangent=None):
        A = torch.as_tensor(A0, **F32).requires_grad_(True)
        c = torch.as_tensor(inp["coeffs"], **F32).requires_grad_(True)
        flat = torch.as_tensor(inp["flat"], **F32).requires_grad_(True)
        optics = dl.AngularOpticalSystem(512, 1.0, [dl.TransmissiveLayer(A, normalise=True),
                                                    dl.BasisLayer(B, c)], 256, 0.02, 1)
        det = dl.LayeredDetector([dl.ApplyPixelResponse(flat)])
        img = det.model(optics.propagate(inp["wavelengths"], return_psf=True))
        m = img * scale
        loss = (m - torch.as_tensor(r["data"], **F32) * torch.log(m)).sum()
        if cotangent is None:
            loss.backward()
        else:
            img.backward(torch.as_tensor(cotangent, **F32))
        return (img.detach().cpu().numpy(), float(loss), c.grad.cpu().numpy(),
                A.grad.cpu().numpy(), flat.grad.cpu().numpy())

    img, loss, gc_e2e, _, _ = run()
    e_img = rel(img, r["image"])
    e_loss = abs(loss - float(r["loss"])) / abs(float(r["loss"]))
    e_e2e = rel(gc_e2e, r["grad_c"])
    # dL/dimage at the reference image (FP64 oracle)
    To, Bo = O.circular_aperture(512, 1.0, oversample=1, secondary_diameter=0.1,
                                 zernike_nolls=inp["nolls"])
    L = len(inp["wavelengths"])
    img_ref = O.poly_psf(To * (1.0 + inp["amp_pert"]), O.eval_basis(Bo, inp["coeffs"]),
                         inp["wavelengths"], np.full(L, 1.0 / L), 1.0, 256,
                         0.02 * RI.ARCSEC) * inp["flat"]
    assert rel(img_ref, r["image"]) < 1e-6
    g_img = scale * (1.0 - data_np / (scale * img_ref))
    _, _, gc, ga, gf = run(g_img)
    e_c = rel(gc, r["grad_c"])
    print(f"cfg3 {variant}: image {e_img:.2e}, loss {e_loss:.2e}, coefficient gradient "
          f"{e_c:.2e} (reference cotangent), end-to-end {e_e2e:.2e}")
    assert e_img < 1e-5 and e_loss < 1e-5 and e_c < 1e-5 and e_e2e < 1e-4
    for v, d in zip(inp["dir_amp"], r["dd_amp"]):
        assert dd_ok(ga, v * Tn, float(d))
    for v, d in zip(inp["dir_flat"], r["dd_flat"]):
        assert dd_ok(gf, v, float(d))


@pytest.mark.parametrize("variant", VARIANTS, indirect=True)
def test_cfg4_point_sources_match_dlux(cuda, variant):
    """Config 4's pupil, focal and wavelength sizes (1024^2 -> 128^2, 16 wavelengths)
    with 4 sources: image, and directional derivatives w.r.t. positions and fluxes."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    r, inp = load("cfg4"), RI.cfg4()
    T, B = dlu.circular_aperture(1024, 1.0, oversample=1, secondary_diameter=0.1,
                                 zernike_nolls=inp["nolls"])
    c = torch.as_tensor(inp["coeffs"], **F32)
    optics = dl.AngularOpticalSystem(1024, 1.0, [dl.TransmissiveLayer(T, normalise=True),
                                                 dl.BasisLayer(B, c)], 128, 0.02, 1)
    pos = torch.as_tensor(inp["positions"], dtype=torch.float64).requires_grad_(True)
    flux = torch.as_tensor(inp["fluxes"], **F32).requires_grad_(True)
    img = dl.PointSources(inp["wavelengths"], position=pos, flux=flux).model(optics)
    loss = (img * torch.as_tensor(inp["R"], **F32)).sum()
    loss.backward()
    e_img = rel(img.detach().cpu().numpy(), r["image"])
    print(f"cfg4 {variant}: image {e_img:.2e}")
    assert e_img < 1e-5
    gp = pos.grad.cpu().numpy()
    for v, d in zip(inp["dir_pos"] / RI.ARCSEC, r["dd_pos"]):
        assert dd_ok(gp, v, float(d))
    gfl = flux.grad.cpu().numpy()
    for v, d in zip(inp["dir_flux"], r["dd_flux"]):
        assert dd_ok(gfl, v, float(d))
