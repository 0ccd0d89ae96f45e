"""Phase-retrieval gradients (Poisson NLL) through the public API vs FP64 central differences.

The phase-retrieval configuration: per-pixel pupil amplitude 1 + N(0, 0.01)
inside the aperture, Zernike coefficients N(0, 40 nm), a detector with a
per-pixel flat field 1 + N(0, 0.02), data = a Poisson draw of the PSF scaled
to 1e6 photons, loss = sum(m - d log m). It runs here at a reduced size
(128^2 pupil, 64^2 detector, 4 wavelengths) so the FP64 oracle's central
differences finish in seconds. Tolerance: relative error <= 1e-3 against the
central differences (their own truncation error is ~1e-6), <= 1e-4 against
the analytic FP64 reverse pass.
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
        # coefficients: central differences in FP64
        h = 1e-10
        fd = []
        for k in range(len(s["c"])):
            e = np.zeros_like(s["c"])
            e[k] = h
            fd.append((oracle_loss(s, c=s["c"] + e) - oracle_loss(s, c=s["c"] - e)) / (2 * h))
        fd = np.array(fd)
        gc = c.grad.cpu().numpy()
        assert np.linalg.norm(gc - fd) / np.linalg.norm(fd) < 1e-3
        # amplitude and flat: a few pixels
        for (i, j) in [(64, 64 + 20), (30, 70), (100, 60)]:
            e = np.zeros_like(s["A"])
            e[i, j] = 1e-5
            fd_a = (oracle_loss(s, A=s["A"] + e) - oracle_loss(s, A=s["A"] - e)) / 2e-5
            assert abs(A.grad[i, j].item() - fd_a) < 2e-3 * abs(fd_a) + 1e-6 * np.abs(fd).max()
        for (i, j) in [(32, 32), (20, 40)]:
            e = np.zeros_like(s["flat"])
            e[i, j] = 1e-6
            fd_f = (oracle_loss(s, flat=s["flat"] + e) - oracle_loss(s, flat=s["flat"] - e)) / 2e-6
            assert abs(flat.grad[i, j].item() - fd_f) < 1e-3 * abs(fd_f) + 1e-3
    finally:
        dl.set_variant(None)
