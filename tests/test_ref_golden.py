"""The oracle and the host-side builders against fixtures made by dLux itself.

tests/golden/ref_*.npz hold outputs of dLux v0.16.0's own, unmodified code,
run in float64 by tests/golden/make_ref_golden.py (dLux as it runs with
jax_enable_x64). Gradients in them are fourth-order central differences of
dLux's own forward pass. These tests pin the oracle (the FP64 restatement the
CUDA path is checked against everywhere else) to those outputs, and check the
package's host-side setup code (aperture and Zernike basis builders, FFT
sampling and ramps) against them. Transform outputs are stored as complex64,
so the oracle comparisons hold to the storage precision (relative L2 <= 1e-6);
the float64 fixtures (system PSFs, losses and gradients) hold to 1e-9 or to
the differences' own accuracy (1e-7).
"""

import os
import sys

import numpy as np
import pytest

from oracle import dlux_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)
import ref_inputs as RI  # noqa: E402


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def ref():
    return np.load(os.path.join(GOLDEN, "ref_utils.npz"))


def _load(name):
    path = os.path.join(GOLDEN, f"ref_{name}.npz")
    if not os.path.exists(path):
        pytest.skip(f"{path} not generated")
    return np.load(path)


@pytest.mark.parametrize("case", RI.MFT_CASES, ids=[c[0] for c in RI.MFT_CASES])
def test_oracle_mft_matches_dlux(ref, case):
    name, n_in, n_out, ps_in, ps_out, fl, shift, pixel, inv, wl = case
    E = RI.case_field(name, n_in)
    got = O.mft(E, wl, ps_in, n_out, ps_out, fl, shift, pixel, inv)
    assert rel(got, ref[f"mft_{name}"]) < 1e-6
    nf = O.calc_nfringes(wl, n_in, ps_in, n_out, ps_out, fl)
    assert abs(nf - float(ref[f"nfringes_{name}"])) <= 1e-12 * abs(nf)
    if f"tm_{name}" in ref:
        tm = O.transfer_matrix(wl, n_in, ps_in, n_out, ps_out, shift[0], fl, 0.0, inv)
        assert rel(tm, ref[f"tm_{name}"]) < 1e-6


@pytest.mark.parametrize("case", RI.FFT_CASES, ids=[c[0] for c in RI.FFT_CASES])
def test_oracle_fft_matches_dlux(ref, case):
    name, n, ps, wl, fl, pad, inv = case
    E = RI.case_field(name, n, salt=7)
    got, ps_out = O.fft_prop(E, wl, ps, fl, pad, inv)
    assert rel(got, ref[f"fft_{name}"]) < 1e-6
    assert abs(ps_out - float(ref[f"fft_ps_{name}"])) <= 1e-12 * abs(ps_out)
    d, c = O.fft_spec(n * pad, ps, wl, fl)
    assert np.allclose([d, c], ref[f"fft_spec_{name}"], rtol=1e-12, atol=0)


def test_host_fft_spec_and_ramps_match_dlux(ref):
    import dlux_gb300.utils as dlu
    for name, n, ps, wl, fl, pad, inv in RI.FFT_CASES:
        d, c = dlu.fft_spec(n * pad, ps, wl, fl)
        assert np.allclose([d, c], ref[f"fft_spec_{name}"], rtol=1e-12, atol=0)
    xs = np.linspace(-0.5, 0.5, 17)
    for inv in (False, True):
        got = dlu.fft_phase_ramp(xs, 1e-6, 0.3e-6, focal_length=2.0, inverse=inv)
        assert rel(got.numpy(), ref[f"ramp_{int(inv)}"]) < 1e-6


def test_oracle_and_host_zernike_basis_match_dlux(ref):
    import dlux_gb300.utils as dlu
    coords = O.pixel_coords(48, 1.0)
    want = ref["zernike_basis_48"]
    assert rel(O.zernike_basis(list(range(1, 40)), coords, 1.0), want) < 1e-6
    host = dlu.zernike_basis(list(range(1, 40)), coords, 1.0, as_numpy=True)
    assert rel(host, want) < 1e-6


@pytest.mark.parametrize("name", ["cfg1", "cfg2"])
def test_oracle_and_host_apertures_match_dlux(ref, name):
    import dlux_gb300.utils as dlu
    kw = {"cfg1": dict(oversample=1, secondary_diameter=0.1, zernike_nolls=list(range(4, 14))),
          "cfg2": dict(oversample=5, secondary_diameter=0.1, spider_width=0.01,
                       spider_angles=(0, 90, 180, 270), zernike_nolls=list(range(4, 25)))}[name]
    n = {"cfg1": 256, "cfg2": 512}[name]
    step = n // 64
    for T, B in (O.circular_aperture(n, 1.0, **kw), dlu.circular_aperture(n, 1.0, **kw)):
        T = T.cpu().numpy() if hasattr(T, "cpu") else np.asarray(T)
        B = B.cpu().numpy() if hasattr(B, "cpu") else np.asarray(B)
        assert rel(T, ref[f"aperture_T_{name}"]) < 1e-6
        assert rel(B[:, ::step, ::step], ref[f"aperture_Bsub_{name}"]) < 1e-6
        assert rel(B.astype(np.float64).sum((1, 2)), ref[f"aperture_Bsum_{name}"]) < 1e-5
        assert rel((B.astype(np.float64) ** 2).sum((1, 2)), ref[f"aperture_Bsq_{name}"]) < 1e-6


def test_oracle_downsample_and_eval_basis_match_dlux(ref):
    x = RI.normal(np.random.default_rng(9), (64, 64))
    assert rel(O.downsample(x, 4, mean=False), ref["downsample_sum"]) < 1e-12
    assert rel(O.downsample(x, 4, mean=True), ref["downsample_mean"]) < 1e-12
    basis = RI.normal(np.random.default_rng(10), (5, 16, 16))
    coeffs = RI.normal(np.random.default_rng(11), 5)
    assert rel(O.eval_basis(basis, coeffs), ref["eval_basis"]) < 1e-12


def test_oracle_cfg1_psf_and_gradient_match_dlux():
    r = _load("cfg1")
    inp = RI.cfg1()
    T, B = O.circular_aperture(256, 1.0, oversample=1, secondary_diameter=0.1,
                               zernike_nolls=inp["nolls"])
    opd = O.eval_basis(B, inp["coeffs"])
    psf = O.poly_psf(T, opd, inp["wavelengths"], [1.0], 1.0, 128, 0.02 * RI.ARCSEC)
    assert rel(psf, r["psf"]) < 1e-9
    Teff = T / np.sqrt((T ** 2).sum())
    g = O.poly_psf_grad(Teff, opd, inp["wavelengths"], [1.0], 1.0, 128, 0.02 * RI.ARCSEC,
                        inp["R"])
    gc = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))
    assert rel(gc, r["grad"]) < 1e-7


def test_oracle_unaligned_system_matches_dlux():
    """100^2 pupil -> 67^2 PSF, 4 wavelengths: sides that are not multiples of 8."""
    r = _load("unaligned")
    inp = RI.unaligned()
    T, B = O.circular_aperture(100, 1.0, oversample=1, secondary_diameter=0.1,
                               zernike_nolls=inp["nolls"])
    opd = O.eval_basis(B, inp["coeffs"])
    wls, w = inp["wavelengths"], inp["weights"]
    psf = O.poly_psf(T, opd, wls, w, 1.0, 67, 0.03 * RI.ARCSEC)
    assert rel(psf, r["psf"]) < 1e-9
    Teff = T / np.sqrt((T ** 2).sum())
    g = O.poly_psf_grad(Teff, opd, wls, w, 1.0, 67, 0.03 * RI.ARCSEC, inp["R"])
    gc = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))
    assert rel(gc, r["grad"]) < 1e-7


def test_oracle_cfg2_image_and_gradient_match_dlux():
    r = _load("cfg2")
    inp = RI.cfg2()
    T, B = O.circular_aperture(512, 1.0, oversample=5, secondary_diameter=0.1,
                               spider_width=0.01, spider_angles=(0, 90, 180, 270),
                               zernike_nolls=inp["nolls"])
    opd = O.eval_basis(B, inp["coeffs"])
    ps = 0.02 / 4 * RI.ARCSEC
    wls, w = inp["wavelengths"], inp["weights"]
    img = O.downsample(O.poly_psf(T, opd, wls, w, 1.0, 512, ps), 4, mean=False)
    assert rel(img, r["image"]) < 1e-9
    Teff = T / np.sqrt((T ** 2).sum())
    g = O.poly_psf_grad(Teff, opd, wls, w, 1.0, 512, ps, np.kron(inp["R"], np.ones((4, 4))))
    gc = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))
    assert rel(gc, r["grad"]) < 1e-7


@pytest.mark.parametrize("case", RI.APERTURE_SHAPES, ids=[c[0] for c in RI.APERTURE_SHAPES])
def test_oracle_aperture_shapes_match_dlux(case):
    r = _load("apertures")
    name, _, _, oshape = case
    inp = RI.apertures()
    trans, opd, _ = O.aberrated_aperture(oshape, 128, 1.0, RI.APERTURE_NOLLS, inp["coeffs"],
                                         RI.APERTURE_TRANSFORM, 1.5)
    assert rel(trans, r[f"{name}_trans"]) < 1e-6
    assert rel(opd, r[f"{name}_opd"]) < 1e-6
