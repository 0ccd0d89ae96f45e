"""Phase-retrieval gradients (Poisson NLL) through the public API vs the FP64 oracle.

The phase-retrieval configuration: per-pixel pupil amplitude 1 + N(0, 0.01)
inside the aperture, Zernike coefficients N(0, 40 nm), a detector with a
per-pixel flat field 1 + N(0, 0.02), data = a Poisson draw of the PSF scaled
to 1e6 photons, loss = sum(m - d log m). It runs here at a reduced size
(128^2 pupil, 64^2 detector, 4 wavelengths); tests/test_gpu_ref_golden.py runs
the full-size configuration against dLux's own outputs. Every gradient is
compared with the oracle's analytic reverse pass (coefficients, amplitude and
flat field over all pixels, relative L2 <= 1e-5), and the coefficient
gradient also with fourth-order central differences of the oracle in FP64
(relative L2 <= 1e-5; their truncation is ~1e-9).
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu


def setup(seed=3):
    rng = np.random.default_rng(seed)
    n, m, L, nz = 128, 64, 4, 12
    T, B = O.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 4 + nz)))
    A = T * (1 + rng.normal(0, 0.01, T.shape))
    c = rng.normal(0, 40e-9, nz)
    wls = np.linspace(0.9e-6, 1.1e-6, L)
    flat = 1 + rng.normal(0, 0.02, (m, m))
    ps = float(O.arcsec2rad(0.04))
    psf = O.poly_psf(A, O.eval_basis(B, c), wls, np.ones(L) / L, 1.0, m, ps)
    scale = 1e6 / (psf * flat).sum()
    data = rng.poisson(psf * flat * scale).astype(float)
    return dict(n=n, m=m, L=L, A=A, B=B, c=c, wls=wls, flat=flat, ps=ps, scale=scale, data=data)


def oracle_loss(s, A=None, c=None, flat=None):
    A = s["A"] if A is None else A
    c = s["c"] if c is None else c
    flat = s["flat"] if flat is None else flat
    psf = O.poly_psf(A, O.eval_basis(s["B"], c), s["wls"], np.ones(s["L"]) / s["L"], 1.0,
                     s["m"], s["ps"])
    mod = s["scale"] * psf * flat
    return float((mod - s["data"] * np.log(mod)).sum())


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_poisson_nll_gradients(cuda, variant):
    import dlux_gb300 as dl
    dl.set_variant(variant)
    try:
        s = setup()
        dev = "cuda"
        A = torch.as_tensor(s["A"], dtype=torch.float32, device=dev).requires_grad_(True)
        c = torch.as_tensor(s["c"], dtype=torch.float32, device=dev).requires_grad_(True)
        flat = torch.as_tensor(s["flat"], dtype=torch.float32, device=dev).requires_grad_(True)
        B = torch.as_tensor(s["B"], dtype=torch.float32, device=dev)
        optics = dl.AngularOpticalSystem(s["n"], 1.0, [dl.TransmissiveLayer(A, normalise=True),
                                                       dl.BasisLayer(B, c)], s["m"], 0.04)
        det = dl.LayeredDetector([dl.ApplyPixelResponse(flat)])
        src = dl.PointSource(s["wls"])
        img = dl.Telescope(optics, src, det).model()
        mod = s["scale"] * img
        d = torch.as_tensor(s["data"], dtype=torch.float32, device=dev)
        loss = (mod - d * torch.log(mod)).sum()
        loss.backward()
        # value
        assert abs(loss.item() - oracle_loss(s)) < 1e-5 * abs(oracle_loss(s)) + 1e-2
        # analytic FP64 reverse pass: dL/dpsf = scale (1 - d / m) flat, then the chain
        # through the amplitude normalisation A / ||A||
        wls, L, m_ = s["wls"], s["L"], s["m"]
        opd = O.eval_basis(s["B"], s["c"])
        w = np.ones(L) / L
        psf = O.poly_psf(s["A"], opd, wls, w, 1.0, m_, s["ps"])
        mod_ref = s["scale"] * psf * s["flat"]
        G = s["scale"] * (1.0 - s["data"] / mod_ref) * s["flat"]
        nrm = np.sqrt((s["A"] ** 2).sum())
        g = O.poly_psf_grad(s["A"] / nrm, opd, wls, w, 1.0, m_, s["ps"], G)
        gc_ref = np.tensordot(s["B"], g["g_opd"], axes=((1, 2), (0, 1)))
        gA_ref = g["g_amp"] / nrm - s["A"] * (g["g_amp"] * s["A"]).sum() / nrm ** 3
        gF_ref = s["scale"] * (1.0 - s["data"] / mod_ref) * psf
        gc = c.grad.cpu().numpy()
        errs = {"coefficients": np.linalg.norm(gc - gc_ref) / np.linalg.norm(gc_ref),
                "amplitude": np.linalg.norm(A.grad.cpu().numpy() - gA_ref) /
                np.linalg.norm(gA_ref),
                "flat": np.linalg.norm(flat.grad.cpu().numpy() - gF_ref) / np.linalg.norm(gF_ref)}
        # coefficients again: fourth-order central differences of the oracle in FP64
        h = 2e-10
        fd = []
        for k in range(len(s["c"])):
            e = np.zeros_like(s["c"])
            e[k] = h
            fd.append((-oracle_loss(s, c=s["c"] + 2 * e) + 8 * oracle_loss(s, c=s["c"] + e)
                       - 8 * oracle_loss(s, c=s["c"] - e) + oracle_loss(s, c=s["c"] - 2 * e))
                      / (12 * h))
        fd = np.array(fd)
        errs["coefficients_fd"] = np.linalg.norm(gc - fd) / np.linalg.norm(fd)
        print(f"phase retrieval {variant}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
        for k, v in errs.items():
            assert v < 1e-5, (k, v)
    finally:
        dl.set_variant(None)
