"""Phase-retrieval gradients (Poisson NLL) through the public API vs the FP64 oracle.

The phase-retrieval configuration: per-pixel pupil amplitude 1 + N(0, 0.01)
inside the aperture, Zernike coefficients N(0, 40 nm), a detector with a
per-pixel flat field 1 + N(0, 0.02), data = a Poisson draw of the PSF scaled
to 1e6 photons, loss = sum(m - d log m). It runs here at a reduced size
(128^2 pupil, 64^2 detector, 4 wavelengths); tests/test_gpu_ref_golden.py runs
the full-size configuration against dLux's own outputs.

The NLL's cotangent dL/dm = 1 - d/m is a difference of nearly equal terms
near the data (d ~ m +- sqrt(m)), so it magnifies the model image's relative
error by up to ~sqrt(counts) (~1e2 here): an image within 1e-6 of the oracle
gives an end-to-end gradient within ~1e-5 to 1e-4. The reverse kernels are
therefore checked on the oracle's own cotangent: the image is backpropagated
with dL/dimage evaluated at the FP64 oracle's image, and the coefficient,
amplitude and flat-field gradients (all pixels) must be within 1e-5
(relative L2) of the oracle's analytic reverse pass, the coefficient
gradient also of fourth-order central differences of the oracle in FP64
(truncation ~1e-9). The end-to-end autograd gradient is reported and held to
1e-4, the conditioning bound above.
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
        wls, L, m_ = s["wls"], s["L"], s["m"]
        w = np.ones(L) / L
        opd = O.eval_basis(s["B"], s["c"])
        psf_ref = O.poly_psf(s["A"], opd, wls, w, 1.0, m_, s["ps"])
        mod_ref = s["scale"] * psf_ref * s["flat"]
        # dL/dimage at the oracle's image, and the oracle's analytic reverse pass
        g_img = s["scale"] * (1.0 - s["data"] / mod_ref)
        G = g_img * s["flat"]                                   # dL/dpsf
        nrm = np.sqrt((s["A"] ** 2).sum())
        g = O.poly_psf_grad(s["A"] / nrm, opd, wls, w, 1.0, m_, s["ps"], G)
        gc_ref = np.tensordot(s["B"], g["g_opd"], axes=((1, 2), (0, 1)))
        gA_ref = g["g_amp"] / nrm - s["A"] * (g["g_amp"] * s["A"]).sum() / nrm ** 3
        gF_ref = g_img * psf_ref

        def run(cotangent=None):
            A = torch.as_tensor(s["A"], dtype=torch.float32, device=dev).requires_grad_(True)
            c = torch.as_tensor(s["c"], dtype=torch.float32, device=dev).requires_grad_(True)
            flat = torch.as_tensor(s["flat"], dtype=torch.float32,
                                   device=dev).requires_grad_(True)
            B = torch.as_tensor(s["B"], dtype=torch.float32, device=dev)
            optics = dl.AngularOpticalSystem(s["n"], 1.0,
                                             [dl.TransmissiveLayer(A, normalise=True),
                                              dl.BasisLayer(B, c)], s["m"], 0.04)
            det = dl.LayeredDetector([dl.ApplyPixelResponse(flat)])
            img = dl.Telescope(optics, dl.PointSource(s["wls"]), det).model()
            mod = s["scale"] * img
            d = torch.as_tensor(s["data"], dtype=torch.float32, device=dev)
            loss = (mod - d * torch.log(mod)).sum()
            if cotangent is None:
                loss.backward()
            else:
                img.backward(torch.as_tensor(cotangent, dtype=torch.float32, device=dev))
            return (loss.item(), c.grad.cpu().numpy(), A.grad.cpu().numpy(),
                    flat.grad.cpu().numpy())

        def rel(a, b):
            return float(np.linalg.norm(a - b) / np.linalg.norm(b))

        loss, gc_e2e, _, _ = run()
        assert abs(loss - oracle_loss(s)) < 1e-5 * abs(oracle_loss(s))
        _, gc, gA, gF = run(g_img)
        errs = {"coefficients": rel(gc, gc_ref), "amplitude": rel(gA, gA_ref),
                "flat": rel(gF, gF_ref)}
        # coefficients again: fourth-order central differences of the oracle in FP64,
        # with the data term's cotangent held at the oracle's image (a linear functional)
        h = 2e-10
        fd = []
        for k in range(len(s["c"])):
            e = np.zeros_like(s["c"])
            e[k] = h

            def lin(cc):
                p = O.poly_psf(s["A"], O.eval_basis(s["B"], cc), wls, w, 1.0, m_, s["ps"])
                return float((G * p).sum())
            fd.append((-lin(s["c"] + 2 * e) + 8 * lin(s["c"] + e) - 8 * lin(s["c"] - e)
                       + lin(s["c"] - 2 * e)) / (12 * h))
        fd = np.array(fd)
        errs["coefficients_fd"] = rel(gc, fd)
        e2e = rel(gc_e2e, gc_ref)
        print(f"phase retrieval {variant}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items())
              + f"; end-to-end coefficient gradient {e2e:.2e}")
        for k, v in errs.items():
            assert v < 1e-5, (k, v)
        assert e2e < 1e-4
    finally:
        dl.set_variant(None)
