"""Every layer type, through the public API, against outputs made by dLux itself.

tests/golden/ref_layers.npz holds PSFs, losses sum(R * PSF) and their gradients
from dLux v0.16.0's own classes (run in float64 by tests/golden/make_ref_golden.py;
gradients are fourth-order central differences of dLux's forward): Optic and
BasisOptic (layers/optics.py:17-175), AberratedLayer, BasisLayer effects "phase"
and "amplitude", Tilt and Normalise (layers/optical_layers.py:189-371),
CartesianOpticalSystem (optical_systems.py:683-775), a LayeredOpticalSystem
with an MFT layer (the layer-by-layer path: phasor kernel and its reverse
kernel, MFT plans, weighted intensity kernel), and Wavefront.normalise in
"power" and "peak" mode (wavefronts.py:397-424).

Tolerances: PSFs, phasors and gradient vectors relative L2 <= 1e-5 in both
arithmetic forms; a directional derivative d = sum g v along the fixture's
seeded direction v as |d - d_ref| <= 1e-5 (|d_ref| + ||g * v||_2).
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

F32 = dict(dtype=torch.float32, device="cuda")
VARIANTS = ["split_bf16", "fp32"]


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def dd_ok(g, v, d_ref, tol=1e-5):
    g = np.asarray(g, np.float64)
    v = np.asarray(v, np.float64)
    d = float((g * v).sum())
    scale = abs(d_ref) + float(np.linalg.norm(g * v))
    print(f"  directional derivative {d:.6e} vs dLux {d_ref:.6e}: "
          f"{abs(d - d_ref) / scale:.2e} of scale")
    return abs(d - d_ref) <= tol * scale


@pytest.fixture(scope="module")
def setup():
    import dlux_gb300.utils as dlu
    inp = RI.layers()
    T, B = dlu.circular_aperture(64, 1.0, oversample=3, secondary_diameter=0.1,
                                 zernike_nolls=inp["nolls"])
    Tn = T.cpu().numpy().astype(np.float64)
    A = Tn * (1.0 + inp["amp_pert"])
    return inp, Tn, A, B, np.load(os.path.join(GOLDEN, "ref_layers.npz"))


@pytest.fixture
def variant(request):
    import dlux_gb300 as dl
    dl.set_variant(request.param)
    yield request.param
    dl.set_variant(None)


def _systems(dl, inp, A, B):
    """name -> (builder taking the differentiated input, initial value, kind)."""
    At = torch.as_tensor(A, **F32)
    opd0 = torch.as_tensor(inp["opd"], **F32)
    ph0 = torch.as_tensor(inp["phase"], **F32)
    c0 = torch.as_tensor(inp["coeffs"], **F32)
    ps = 0.04 * RI.ARCSEC

    def ang(layers):
        return dl.AngularOpticalSystem(64, 1.0, layers, 32, 0.04, 1)

    return {
        "optic": (lambda o: ang([dl.Optic(At, o, ph0, normalise=True)]), opd0, "dir_opd"),
        "optic_phase": (lambda p: ang([dl.Optic(At, opd0, p, normalise=True)]), ph0,
                        "dir_phase"),
        "optic_amp": (lambda a: ang([dl.Optic(a, opd0, None, normalise=True)]), At, "dir_amp"),
        "basis_optic": (lambda c: ang([dl.BasisOptic(B, At, c, normalise=True)]), c0, "grad"),
        "aberrated_opd": (lambda o: ang([dl.TransmissiveLayer(At, normalise=True),
                                         dl.AberratedLayer(opd=o)]), opd0, "dir_opd"),
        "aberrated_phase": (lambda p: ang([dl.TransmissiveLayer(At, normalise=True),
                                           dl.AberratedLayer(phase=p)]), ph0, "dir_phase"),
        "basis_phase": (lambda c: ang([dl.TransmissiveLayer(At, normalise=True),
                                       dl.BasisLayer(B, c * 1e7, effect="phase")]), c0, "grad"),
        "basis_amplitude": (lambda c: ang([dl.TransmissiveLayer(At),
                                           dl.BasisLayer(B, c * 1e6, effect="amplitude"),
                                           dl.Normalise()]), c0, "grad"),
        "tilt_layer": (lambda t: ang([dl.TransmissiveLayer(At, normalise=True), dl.Tilt(t),
                                      dl.BasisLayer(B, c0)]),
                       torch.as_tensor(inp["tilt"], dtype=torch.float64), "grad"),
        "normalise_layer": (lambda c: ang([dl.TransmissiveLayer(At), dl.BasisLayer(B, c),
                                           dl.Normalise()]), c0, "grad"),
        "cartesian": (lambda c: dl.CartesianOpticalSystem(
            64, 1.0, [dl.TransmissiveLayer(At, normalise=True), dl.BasisLayer(B, c)], 5.0, 32,
            0.8, 1), c0, "grad"),
        "layered_mft": (lambda c: dl.LayeredOpticalSystem(
            64, 1.0, [dl.TransmissiveLayer(At, normalise=True), dl.BasisLayer(B, c),
                      dl.MFT(32, ps)]), c0, "grad"),
    }


NAMES = ["optic", "optic_phase", "optic_amp", "basis_optic", "aberrated_opd", "aberrated_phase",
         "basis_phase", "basis_amplitude", "tilt_layer", "normalise_layer", "cartesian",
         "layered_mft"]


@pytest.mark.parametrize("variant", VARIANTS, indirect=True)
@pytest.mark.parametrize("name", NAMES)
def test_layer_type_matches_dlux(cuda, setup, variant, name):
    import dlux_gb300 as dl
    inp, Tn, A, B, ref = setup
    make, x0, kind = _systems(dl, inp, A, B)[name]
    x = x0.detach().clone().requires_grad_(True)
    psf = make(x).propagate(inp["wavelengths"], weights=torch.as_tensor(inp["weights"], **F32))
    loss = (psf * torch.as_tensor(inp["R"], **F32)).sum()
    loss.backward()
    e_psf = rel(psf.detach().cpu().numpy(), ref[f"{name}_psf"])
    print(f"{name} {variant}: PSF {e_psf:.2e}")
    assert e_psf < 1e-5
    g = x.grad.detach().cpu().numpy()
    if kind == "grad":
        e_g = rel(g, ref[f"{name}_grad"])
        print(f"  gradient {e_g:.2e}")
        assert e_g < 1e-5
    else:
        v = inp[kind] * (Tn if kind == "dir_amp" else 1.0)
        assert dd_ok(g, v, float(ref[f"{name}_dd"]))


@pytest.mark.parametrize("variant", VARIANTS, indirect=True)
def test_wavefront_normalise_power_and_peak_match_dlux(cuda, setup, variant):
    """Wavefront.normalise on its own, and "peak" normalisation between the aperture
    and the MFT with the gradient of the loss w.r.t. the OPD through it."""
    import dlux_gb300 as dl
    inp, Tn, A, B, ref = setup
    At = torch.as_tensor(A, **F32)
    opd0 = torch.as_tensor(inp["opd"], **F32)
    wf = dl.Wavefront(1.0e-6, 64, diameter=1.0) * At
    assert rel(wf.add_opd(opd0).normalise("power").phasor.cpu().numpy(),
               ref["power_phasor"]) < 1e-5
    assert rel(wf.add_opd(opd0).normalise("peak", 2.0).phasor.cpu().numpy(),
               ref["peak_phasor"]) < 1e-5
    with pytest.raises(ValueError, match="power"):
        wf.normalise("energy")
    o = opd0.detach().clone().requires_grad_(True)
    w2 = (dl.Wavefront(1.0e-6, 64, diameter=1.0) * At).add_opd(o).normalise("peak")
    psf = w2.propagate(32, 0.04 * RI.ARCSEC).psf
    (psf * torch.as_tensor(inp["R"], **F32)).sum().backward()
    assert rel(psf.detach().cpu().numpy(), ref["peak_psf"]) < 1e-5
    assert dd_ok(o.grad.cpu().numpy(), inp["dir_opd"], float(ref["peak_dd"]))


def test_layer_path_reverse_kernels_are_deterministic(cuda, setup):
    """The layer-by-layer reverse pass (phasor, intensity and normalisation kernels)
    gives bit-identical gradients on repeated runs."""
    import dlux_gb300 as dl
    inp, Tn, A, B, ref = setup
    make, x0, _ = _systems(dl, inp, A, B)["layered_mft"]
    grads = []
    for _ in range(2):
        x = x0.detach().clone().requires_grad_(True)
        psf = make(x).propagate(inp["wavelengths"])
        (psf * torch.as_tensor(inp["R"], **F32)).sum().backward()
        grads.append(x.grad.cpu().numpy())
    assert np.array_equal(grads[0], grads[1])
