"""Golden fixtures made by dLux itself (tests/golden/ref_*.npz).

Runs dLux's own, unmodified source (the ``src`` directory of dLux v0.16.0,
passed as the first argument) on the host under the NumPy stand-ins of
ref_standin.py, in float64 -- dLux as it runs with jax_enable_x64 -- and
saves its outputs on the seeded inputs of ref_inputs.py:

  ref_utils.npz  utils functions: transfer_matrix, calc_nfringes and MFT
                 (utils/propagation.py:67-256), FFT (:8-64), fft_spec and
                 fft_phase_ramp (utils/fourier.py:14-78), zernike_basis
                 (utils/zernikes.py:297-315), circular_aperture
                 (utils/apertures.py:153-242), downsample
                 (utils/array_ops.py:124-162), eval_basis (utils/math.py:177-196);
  ref_cfg1.npz   config 1 through AngularOpticalSystem.propagate
                 (optical_systems.py:147-223): PSF and the gradient of
                 sum(R * PSF) with respect to the coefficients;
  ref_unaligned.npz a system with sides that are not multiples of 8 (100^2
                 pupil, 67^2 PSF, 4 wavelengths): PSF and coefficient gradient;
  ref_cfg2.npz   config 2 (the benchmark workload) through
                 AngularOpticalSystem + LayeredDetector([Downsample(4)]):
                 image and coefficient gradient of sum(R * image);
  ref_cfg3.npz   config 3: image through ApplyPixelResponse, the Poisson data
                 and NLL, the coefficient gradient and directional derivatives
                 with respect to the pupil amplitude and the flat field;
  ref_cfg4.npz   config 4 at its sizes with 4 sources, PointSources.model
                 (sources.py:392-411): image, and directional derivatives of
                 sum(R * image) with respect to positions and fluxes;
  ref_layers.npz each layer type of the layer-by-layer path at small size:
                 Optic and BasisOptic (layers/optics.py:17-175), AberratedLayer,
                 BasisLayer effects "phase" and "amplitude", Tilt and Normalise
                 (layers/optical_layers.py:189-371), CartesianOpticalSystem
                 (optical_systems.py:683-775), a LayeredOpticalSystem with an MFT
                 layer, and Wavefront.normalise "power"/"peak"
                 (wavefronts.py:397-424): PSFs, losses and gradients;
  ref_apertures.npz AberratedAperture over Circular, Square, Rectangular and
                 RegPoly apertures (layers/apertures.py:240-800) under a
                 CoordTransform: transmission, OPD (polygon-stretched Zernikes,
                 utils/zernikes.py:318-419, for the polygons) and a system PSF
                 with its coefficient gradient.

dLux's gradients come from JAX autodiff, which cannot run here, so every
gradient is taken by fourth-order central differences of dLux's own forward in
float64 (step h: truncation ~h^4, far below the 1e-5 tolerance of the tests).
The script also checks the oracle (oracle/dlux_oracle.py, FP64) against every
fixture before saving and prints the differences.

    python tests/golden/make_ref_golden.py <dLux src dir> [utils cfg1 unaligned cfg2 ...]
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import ref_inputs as RI  # noqa: E402
import ref_standin  # noqa: E402
from ref_standin import J  # noqa: E402


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def fd4(f, x, v, h):
    """Fourth-order central difference of f at x along v."""
    return (-f(x + 2 * h * v) + 8 * f(x + h * v) - 8 * f(x - h * v) + f(x - 2 * h * v)) / (12 * h)


def fd4_grad(f, x, h):
    g = np.zeros(len(x))
    for i in range(len(x)):
        e = np.zeros(len(x))
        e[i] = 1.0
        g[i] = fd4(f, x, e, h)
    return g


def make_utils(dl, O):
    dlu = dl.utils
    out = {}
    for name, n_in, n_out, ps_in, ps_out, fl, shift, pixel, inv, wl in RI.MFT_CASES:
        E = RI.case_field(name, n_in)
        sh = np.array(shift, float)
        got = dlu.MFT(J(E.copy()), wl, ps_in, n_out, ps_out, focal_length=fl, shift=J(sh.copy()),
                      pixel=pixel, inverse=inv)
        ora = O.mft(E, wl, ps_in, n_out, ps_out, fl, shift, pixel, inv)
        print(f"MFT {name}: oracle vs dLux {rel(ora, got):.2e}")
        out[f"mft_{name}"] = got.astype(np.complex64)
        out[f"nfringes_{name}"] = np.float64(dlu.propagation.calc_nfringes(
            wl, n_in, ps_in, n_out, ps_out, focal_length=fl))
        tm = dlu.propagation.transfer_matrix(wl, n_in, ps_in, n_out, ps_out, shift=sh[0], focal_length=fl,
                                 inverse=inv)
        tora = O.transfer_matrix(wl, n_in, ps_in, n_out, ps_out, sh[0], fl, 0.0, inv)
        print(f"  transfer_matrix: oracle vs dLux {rel(tora, tm):.2e}")
        if n_in * n_out <= 256 * 128:
            out[f"tm_{name}"] = tm.astype(np.complex64)
    for name, n, ps, wl, fl, pad, inv in RI.FFT_CASES:
        E = RI.case_field(name, n, salt=7)
        got, ps_out = dlu.FFT(J(E.copy()), wl, ps, focal_length=fl, pad=pad, inverse=inv)
        ora, ops = O.fft_prop(E, wl, ps, fl, pad, inv)
        print(f"FFT {name}: oracle vs dLux {rel(ora, got):.2e}, pixel scale "
              f"{abs(ops - ps_out) / abs(ps_out):.1e}")
        out[f"fft_{name}"] = got.astype(np.complex64)
        out[f"fft_ps_{name}"] = np.float64(ps_out)
        d, c = dlu.fft_spec(n * pad, ps, wl, focal_length=fl)
        out[f"fft_spec_{name}"] = np.array([d, c], float)
    xs = np.linspace(-0.5, 0.5, 17)
    for inv in (False, True):
        out[f"ramp_{int(inv)}"] = dlu.fft_phase_ramp(xs, 1e-6, 0.3e-6, focal_length=2.0,
                                                     inverse=inv)
    coords = dlu.pixel_coords(48, 1.0)
    zb = dlu.zernike_basis(list(range(1, 40)), coords, 1.0)
    out["zernike_basis_48"] = zb.astype(np.float32)
    print(f"zernike_basis: oracle vs dLux "
          f"{rel(O.zernike_basis(list(range(1, 40)), coords, 1.0), zb):.2e}")
    apertures = {
        "cfg1": dict(npixels=256, oversample=1, secondary_diameter=0.1,
                     zernike_nolls=list(range(4, 14))),
        "cfg2": dict(npixels=512, oversample=5, secondary_diameter=0.1, spider_width=0.01,
                     spider_angles=(0, 90, 180, 270), zernike_nolls=list(range(4, 25))),
    }
    for name, kw in apertures.items():
        n = kw.pop("npixels")
        T, B = dlu.circular_aperture(n, 1.0, **kw)
        To, Bo = O.circular_aperture(n, 1.0, **kw)
        print(f"circular_aperture {name}: T {rel(To, T):.2e}, B {rel(Bo, B):.2e}")
        step = n // 64
        out[f"aperture_T_{name}"] = T.astype(np.float32)
        out[f"aperture_Bsub_{name}"] = B[:, ::step, ::step].astype(np.float32)
        out[f"aperture_Bsum_{name}"] = B.sum((1, 2))
        out[f"aperture_Bsq_{name}"] = (B ** 2).sum((1, 2))
    x = RI.normal(np.random.default_rng(9), (64, 64))
    out["downsample_sum"] = dlu.downsample(x, 4, mean=False)
    out["downsample_mean"] = dlu.downsample(x, 4, mean=True)
    basis = RI.normal(np.random.default_rng(10), (5, 16, 16))
    coeffs = RI.normal(np.random.default_rng(11), 5)
    out["eval_basis"] = dlu.eval_basis(basis, coeffs)
    return out


def _cfg1_system(dl, T, B, c):
    L = dl.layers
    return dl.optical_systems.AngularOpticalSystem(
        256, 1.0, [L.TransmissiveLayer(T, normalise=True), L.BasisLayer(B, c)], 128, 0.02, 1)


def make_cfg1(dl, O):
    inp = RI.cfg1()
    T, B = dl.utils.circular_aperture(256, 1.0, oversample=1, secondary_diameter=0.1,
                                      zernike_nolls=inp["nolls"])
    wls = inp["wavelengths"]

    def psf_of(c):
        return _cfg1_system(dl, T, B, c).propagate(wls)

    psf = psf_of(inp["coeffs"])
    loss = lambda c: float((psf_of(c) * inp["R"]).sum())  # noqa: E731
    grad = fd4_grad(loss, inp["coeffs"], 2e-10)
    ora = O.poly_psf(T, np.tensordot(B, inp["coeffs"], axes=(0, 0)), wls, [1.0], 1.0, 128,
                     0.02 * RI.ARCSEC)
    Teff = T / np.sqrt((T ** 2).sum())
    g = O.poly_psf_grad(Teff, np.tensordot(B, inp["coeffs"], axes=(0, 0)), wls, [1.0], 1.0,
                        128, 0.02 * RI.ARCSEC, inp["R"])
    gc = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))
    print(f"cfg1: PSF oracle vs dLux {rel(ora, psf):.2e}, gradient oracle vs dLux FD "
          f"{rel(gc, grad):.2e}")
    return {"psf": psf, "loss": loss(inp["coeffs"]), "grad": grad}


def make_unaligned(dl, O):
    inp = RI.unaligned()
    L = dl.layers
    T, B = dl.utils.circular_aperture(100, 1.0, oversample=1, secondary_diameter=0.1,
                                      zernike_nolls=inp["nolls"])
    wls, w = inp["wavelengths"], inp["weights"]

    def psf_of(c):
        return dl.optical_systems.AngularOpticalSystem(
            100, 1.0, [L.TransmissiveLayer(T, normalise=True), L.BasisLayer(B, c)], 67,
            0.03, 1).propagate(wls, weights=w)

    psf = psf_of(inp["coeffs"])
    loss = lambda c: float((psf_of(c) * inp["R"]).sum())  # noqa: E731
    grad = fd4_grad(loss, inp["coeffs"], 2e-10)
    opd = np.tensordot(B, inp["coeffs"], axes=(0, 0))
    ora = O.poly_psf(T, opd, wls, w, 1.0, 67, 0.03 * RI.ARCSEC)
    Teff = T / np.sqrt((T ** 2).sum())
    g = O.poly_psf_grad(Teff, opd, wls, w, 1.0, 67, 0.03 * RI.ARCSEC, inp["R"])
    gc = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))
    print(f"unaligned: PSF oracle vs dLux {rel(ora, psf):.2e}, gradient oracle vs dLux FD "
          f"{rel(gc, grad):.2e}")
    return {"psf": psf, "loss": loss(inp["coeffs"]), "grad": grad}


def make_cfg2(dl, O):
    inp = RI.cfg2()
    L = dl.layers
    T, B = dl.utils.circular_aperture(512, 1.0, oversample=5, secondary_diameter=0.1,
                                      spider_width=0.01, spider_angles=(0, 90, 180, 270),
                                      zernike_nolls=inp["nolls"])
    wls, w = inp["wavelengths"], inp["weights"]
    det = dl.detectors.LayeredDetector([L.Downsample(4)])

    def image_of(c):
        optics = dl.optical_systems.AngularOpticalSystem(
            512, 1.0, [L.TransmissiveLayer(T, normalise=True), L.BasisLayer(B, c)], 128,
            0.02, 4)
        return det.model(optics.propagate(wls, weights=w, return_psf=True))

    t0 = time.time()
    img = image_of(inp["coeffs"])
    print(f"cfg2 forward {time.time() - t0:.1f} s")
    loss = lambda c: float((image_of(c) * inp["R"]).sum())  # noqa: E731
    grad = fd4_grad(loss, inp["coeffs"], 2e-10)
    opd = np.tensordot(B, inp["coeffs"], axes=(0, 0))
    ps = 0.02 / 4 * RI.ARCSEC
    ora = O.downsample(O.poly_psf(T, opd, wls, w, 1.0, 512, ps), 4, mean=False)
    Teff = T / np.sqrt((T ** 2).sum())
    G = np.kron(inp["R"], np.ones((4, 4)))
    g = O.poly_psf_grad(Teff, opd, wls, w, 1.0, 512, ps, G)
    gc = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))
    print(f"cfg2: image oracle vs dLux {rel(ora, img):.2e}, gradient oracle vs dLux FD "
          f"{rel(gc, grad):.2e}")
    return {"image": img, "loss": loss(inp["coeffs"]), "grad": grad}


def make_cfg3(dl, O):
    inp = RI.cfg3()
    L = dl.layers
    T, B = dl.utils.circular_aperture(512, 1.0, oversample=1, secondary_diameter=0.1,
                                      zernike_nolls=inp["nolls"])
    A0 = T * (1.0 + inp["amp_pert"])
    wls = inp["wavelengths"]

    def image_of(c, A, flat):
        optics = dl.optical_systems.AngularOpticalSystem(
            512, 1.0, [L.TransmissiveLayer(A, normalise=True), L.BasisLayer(B, c)], 256,
            0.02, 1)
        det = dl.detectors.LayeredDetector([L.ApplyPixelResponse(flat)])
        return det.model(optics.propagate(wls, return_psf=True))

    img = image_of(inp["coeffs"], A0, inp["flat"])
    scale = 1e6 / img.sum()
    lam = img * scale
    # data: a seeded Gaussian stand-in for the Poisson draw, rounded to counts
    z = RI.normal(np.random.default_rng(303), lam.shape)
    data = np.maximum(0.0, np.round(lam + np.sqrt(lam) * z))

    def nll(c, A, flat):
        m = image_of(c, A, flat) * scale
        return float((m - data * np.log(m)).sum())

    c0, f0 = inp["coeffs"], inp["flat"]
    grad_c = fd4_grad(lambda c: nll(c, A0, f0), c0, 2e-10)
    # steps of 1e-4 along N(0, 1) directions: the NLL is ~4e6, so smaller steps lose
    # digits to rounding; the fourth-order truncation at 1e-4 is far below that
    d_amp = [fd4(lambda A: nll(c0, A, f0), A0, v * T, 1e-4) for v in inp["dir_amp"]]
    d_flat = [fd4(lambda f: nll(c0, A0, f), f0, v, 1e-4) for v in inp["dir_flat"]]
    opd = np.tensordot(B, c0, axes=(0, 0))
    ora = O.poly_psf(A0, opd, wls, np.full(len(wls), 1.0 / len(wls)), 1.0, 256,
                     0.02 * RI.ARCSEC) * f0
    print(f"cfg3: image oracle vs dLux {rel(ora, img):.2e}")
    return {"image": img.astype(np.float32), "data": data.astype(np.float32),
            "scale": scale, "loss": nll(c0, A0, f0), "grad_c": grad_c,
            "dd_amp": np.array(d_amp), "dd_flat": np.array(d_flat)}


def make_cfg4(dl, O):
    inp = RI.cfg4()
    L = dl.layers
    T, B = dl.utils.circular_aperture(1024, 1.0, oversample=1, secondary_diameter=0.1,
                                      zernike_nolls=inp["nolls"])
    optics = dl.optical_systems.AngularOpticalSystem(
        1024, 1.0, [L.TransmissiveLayer(T, normalise=True), L.BasisLayer(B, inp["coeffs"])],
        128, 0.02, 1)
    wls = inp["wavelengths"]

    def image_of(pos, flux):
        return dl.sources.PointSources(wls, position=pos, flux=flux).model(optics)

    t0 = time.time()
    img = image_of(inp["positions"], inp["fluxes"])
    print(f"cfg4 forward {time.time() - t0:.1f} s")
    loss_pos = lambda p: float((image_of(p, inp["fluxes"]) * inp["R"]).sum())  # noqa: E731
    loss_flux = lambda f: float((image_of(inp["positions"], f) * inp["R"]).sum())  # noqa: E731
    dd_pos = [fd4(loss_pos, inp["positions"], v, 1e-9) for v in inp["dir_pos"] / RI.ARCSEC]
    dd_flux = [fd4(loss_flux, inp["fluxes"], v, 1.0) for v in inp["dir_flux"]]
    opd = np.tensordot(B, inp["coeffs"], axes=(0, 0))
    w = np.full(len(wls), 1.0 / len(wls))
    ora = sum(f * O.poly_psf(T, opd, wls, w, 1.0, 128, 0.02 * RI.ARCSEC, offset=tuple(p))
              for p, f in zip(inp["positions"], inp["fluxes"]))
    print(f"cfg4: image oracle vs dLux {rel(ora, img):.2e}")
    return {"image": img, "loss": float((img * inp["R"]).sum()), "dd_pos": np.array(dd_pos),
            "dd_flux": np.array(dd_flux)}


def make_layers(dl, O):
    """Each layer type of the layer-by-layer path, through dLux's own classes."""
    inp = RI.layers()
    L = dl.layers
    OS = dl.optical_systems
    T, B = dl.utils.circular_aperture(64, 1.0, oversample=3, secondary_diameter=0.1,
                                      zernike_nolls=inp["nolls"])
    A = T * (1.0 + inp["amp_pert"])
    wls, w, R = inp["wavelengths"], inp["weights"], inp["R"]
    opd0, ph0, c0 = inp["opd"], inp["phase"], inp["coeffs"]
    ang = lambda layers: OS.AngularOpticalSystem(64, 1.0, layers, 32, 0.04, 1)  # noqa: E731

    def loss_of(make):
        return lambda x: float((make(x).propagate(wls, weights=w) * R).sum())

    out = {}
    systems = {
        # name: (builder of the system from its differentiated input, x0, kind, h)
        "optic": (lambda o: ang([L.Optic(A, o, ph0, normalise=True)]), opd0, "dir_opd", 0.05),
        "optic_phase": (lambda p: ang([L.Optic(A, opd0, p, normalise=True)]), ph0, "dir_phase",
                        1e-3),
        "optic_amp": (lambda a: ang([L.Optic(a, opd0, None, normalise=True)]), A, "dir_amp", 1e-4),
        "basis_optic": (lambda c: ang([L.BasisOptic(B, A, c, normalise=True)]), c0, "grad",
                        2e-10),
        "aberrated_opd": (lambda o: ang([L.TransmissiveLayer(A, normalise=True),
                                         L.AberratedLayer(opd=o)]), opd0, "dir_opd", 0.05),
        "aberrated_phase": (lambda p: ang([L.TransmissiveLayer(A, normalise=True),
                                           L.AberratedLayer(phase=p)]), ph0, "dir_phase", 1e-3),
        "basis_phase": (lambda c: ang([L.TransmissiveLayer(A, normalise=True),
                                       L.BasisLayer(B, c * 1e7, effect="phase")]), c0, "grad",
                        2e-10),
        "basis_amplitude": (lambda c: ang([L.TransmissiveLayer(A),
                                           L.BasisLayer(B, c * 1e6, effect="amplitude"),
                                           L.Normalise()]), c0, "grad", 2e-10),
        "tilt_layer": (lambda t: ang([L.TransmissiveLayer(A, normalise=True), L.Tilt(t),
                                      L.BasisLayer(B, c0)]), inp["tilt"], "grad", 1e-9),
        "normalise_layer": (lambda c: ang([L.TransmissiveLayer(A), L.BasisLayer(B, c),
                                           L.Normalise()]), c0, "grad", 2e-10),
        "cartesian": (lambda c: OS.CartesianOpticalSystem(
            64, 1.0, [L.TransmissiveLayer(A, normalise=True), L.BasisLayer(B, c)], 5.0, 32,
            0.8, 1), c0, "grad", 2e-10),
        "layered_mft": (lambda c: OS.LayeredOpticalSystem(
            64, 1.0, [L.TransmissiveLayer(A, normalise=True), L.BasisLayer(B, c),
                      L.MFT(32, 0.04 * RI.ARCSEC)]), c0, "grad", 2e-10),
    }
    # Steps h along each direction: the OPD directions are 1e-8 m fields (h = 0.05:
    # ~5e-10 m, a few milliradians of phase), phase directions N(0, 1) rad (h = 1e-3),
    # transmission directions N(0, 1) T (h = 1e-4), coefficients (h = 2e-10 m).
    for name, (make, x0, kind, h) in systems.items():
        f = loss_of(make)
        out[f"{name}_psf"] = make(x0).propagate(wls, weights=w)
        out[f"{name}_loss"] = f(x0)
        if kind == "grad":
            out[f"{name}_grad"] = fd4_grad(f, np.asarray(x0, float), h)
        else:
            out[f"{name}_dd"] = fd4(f, x0, inp[kind] * (T if kind == "dir_amp" else 1.0), h)
        print(f"layers {name}: loss {out[f'{name}_loss']:.6e}")

    # Wavefront.normalise("peak") between the aperture and the MFT, one wavelength
    def peak_psf(o):
        wf = dl.wavefronts.Wavefront(1.0e-6, 64, diameter=1.0)
        wf = wf * A
        wf = wf.add_opd(o)
        wf = wf.normalise("peak")
        wf = wf.propagate(32, 0.04 * RI.ARCSEC)
        return wf.psf
    out["peak_psf"] = peak_psf(opd0)
    out["peak_dd"] = fd4(lambda o: float((peak_psf(o) * R).sum()), opd0, inp["dir_opd"], 0.05)
    # power normalisation of a wavefront, for comparison
    wf = dl.wavefronts.Wavefront(1.0e-6, 64, diameter=1.0) * A
    out["power_phasor"] = wf.add_opd(opd0).normalise("power").phasor
    out["peak_phasor"] = wf.add_opd(opd0).normalise("peak", 2.0).phasor
    return out


def make_apertures(dl, O):
    """AberratedAperture over each dynamic aperture shape, through dLux's own classes:
    transmission and OPD on a transformed grid, and a system PSF with its coefficient
    gradient."""
    inp = RI.apertures()
    L = dl.layers
    out = {}
    wf = dl.wavefronts.Wavefront(1e-6, 128, diameter=1.0)
    coords, ps = wf.coordinates(), wf.pixel_scale
    for name, cls, args, oshape in RI.APERTURE_SHAPES:
        def make(c):
            tf = dl.coordinates.CoordTransform(**{k: np.asarray(v, float) if k != "rotation"
                                                  else v for k, v in
                                                  RI.APERTURE_TRANSFORM.items()})
            ap = getattr(L, cls)(*args, transformation=tf, softening=1.5)
            return L.AberratedAperture(ap, RI.APERTURE_NOLLS, J(np.array(c, float)))
        ab = make(inp["coeffs"])
        trans = ab.transmission(coords, ps)
        opd = ab.eval_basis(coords)
        ot, oo, _ = O.aberrated_aperture(oshape, 128, 1.0, RI.APERTURE_NOLLS, inp["coeffs"],
                                         RI.APERTURE_TRANSFORM, 1.5)
        print(f"aperture {name}: transmission oracle vs dLux {rel(ot, trans):.2e}, "
              f"OPD {rel(oo, opd):.2e}")
        out[f"{name}_trans"] = trans.astype(np.float32)
        out[f"{name}_opd"] = opd.astype(np.float32)

        def psf_of(c):
            return dl.optical_systems.AngularOpticalSystem(
                128, 1.0, [make(c)], 64, 0.03, 1).propagate(inp["wavelengths"])
        out[f"{name}_psf"] = psf_of(inp["coeffs"])
        out[f"{name}_grad"] = fd4_grad(lambda c: float((psf_of(c) * inp["R"]).sum()),
                                       inp["coeffs"], 2e-10)
    return out


def main():
    src = sys.argv[1]
    which = sys.argv[2:] or ["utils", "cfg1", "unaligned", "cfg2", "cfg3", "cfg4", "layers",
                             "apertures"]
    dl = ref_standin.load_dlux(src)
    from oracle import dlux_oracle as O
    makers = {"utils": make_utils, "cfg1": make_cfg1, "unaligned": make_unaligned,
              "cfg2": make_cfg2, "cfg3": make_cfg3,
              "cfg4": make_cfg4, "layers": make_layers, "apertures": make_apertures}
    for name in which:
        t0 = time.time()
        data = makers[name](dl, O)
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, **data)
        print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB, {time.time() - t0:.0f} s)")


if __name__ == "__main__":
    main()
