"""Every dynamic aperture shape under AberratedAperture against dLux's own outputs.

tests/golden/ref_apertures.npz holds, from dLux v0.16.0's own classes (run in
float64 by tests/golden/make_ref_golden.py), the transmission and OPD of
AberratedAperture over CircularAperture, SquareAperture, RectangularAperture
and RegPolyAperture (6 and 5 sides) under a CoordTransform on a 128^2 grid, and
the PSF of a system holding each with the coefficient gradient of sum(R * PSF)
(fourth-order central differences of dLux's forward). The polygonal shapes use
dLux's polygon-stretched Zernikes. Also checks the device's coefficient
gradient kernel against the oracle's polygon basis.

Tolerances: transmission, OPD, PSF and gradients relative L2 <= 1e-5.
"""

import os
import sys

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)
import ref_inputs as RI  # noqa: E402

F32 = dict(dtype=torch.float32, device="cuda")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _aperture(dl, cls, args):
    tf = dl.CoordTransform(**RI.APERTURE_TRANSFORM)
    return getattr(dl, cls)(*args, transformation=tf, softening=1.5)


@pytest.mark.parametrize("case", RI.APERTURE_SHAPES, ids=[c[0] for c in RI.APERTURE_SHAPES])
def test_aperture_shape_matches_dlux(cuda, case):
    import dlux_gb300 as dl
    name, cls, args, oshape = case
    ref = np.load(os.path.join(GOLDEN, "ref_apertures.npz"))
    inp = RI.apertures()
    c = torch.as_tensor(inp["coeffs"], **F32)
    ab = dl.AberratedAperture(_aperture(dl, cls, args), RI.APERTURE_NOLLS, c)
    trans = ab.aperture.transmission(128, 1.0 / 128)
    opd = ab.eval_basis(128, 1.0 / 128)
    e_t, e_o = rel(trans.cpu(), ref[f"{name}_trans"]), rel(opd.detach().cpu(), ref[f"{name}_opd"])
    # the coefficient gradient kernel against the oracle's basis of this shape
    _, _, basis = O.aberrated_aperture(oshape, 128, 1.0, RI.APERTURE_NOLLS, inp["coeffs"],
                                       RI.APERTURE_TRANSFORM, 1.5)
    g = np.random.default_rng(7).normal(size=(128, 128))
    from dlux_gb300 import kernels
    g_d = kernels.aberrated_aperture_grad(ab.aperture.desc(128, 1.0 / 128), RI.APERTURE_NOLLS,
                                          torch.as_tensor(g, **F32))
    e_g = rel(g_d.cpu(), np.tensordot(basis, g, axes=((1, 2), (0, 1))))
    print(f"{name}: transmission {e_t:.2e}, OPD {e_o:.2e}, gradient kernel {e_g:.2e}")
    assert e_t < 1e-5 and e_o < 1e-5 and e_g < 1e-5


@pytest.mark.parametrize("variant", ["split_bf16", "fp32"])
@pytest.mark.parametrize("case", RI.APERTURE_SHAPES, ids=[c[0] for c in RI.APERTURE_SHAPES])
def test_aperture_shape_in_a_system_matches_dlux(cuda, case, variant):
    import dlux_gb300 as dl
    name, cls, args, _ = case
    ref = np.load(os.path.join(GOLDEN, "ref_apertures.npz"))
    inp = RI.apertures()
    dl.set_variant(variant)
    try:
        c = torch.as_tensor(inp["coeffs"], **F32).requires_grad_(True)
        ab = dl.AberratedAperture(_aperture(dl, cls, args), RI.APERTURE_NOLLS, c)
        psf = dl.AngularOpticalSystem(128, 1.0, [ab], 64, 0.03, 1).propagate(inp["wavelengths"])
        (psf * torch.as_tensor(inp["R"], **F32)).sum().backward()
    finally:
        dl.set_variant(None)
    e_p, e_g = rel(psf.detach().cpu(), ref[f"{name}_psf"]), rel(c.grad.cpu(), ref[f"{name}_grad"])
    print(f"{name} {variant}: PSF {e_p:.2e}, coefficient gradient {e_g:.2e}")
    assert e_p < 1e-5 and e_g < 1e-5


def test_polygon_side_limits(cuda):
    import dlux_gb300 as dl
    with pytest.raises(ValueError, match="sides"):
        dl.RegPolyAperture(2, 0.4).transmission(32, 1.0 / 32)
    with pytest.raises(TypeError):
        dl.AberratedAperture(dl.SquareAperture(0.5, occulting=True), [4])
