"""ABCD propagators on the CPU: ray-transfer matrices, the layer API of
dLux's tests/layers/test_abcd_propagators.py, and the oracle's LCT and ASM
restatements pinned by physics identities.

The reference takes the arithmetic from the unvendored abcdLux package and
its tests pin shapes and errors only, so values are pinned here by
independent identities instead:
- the Fraunhofer LCT equals dLux's MFT up to -i dx / d_out;
- ASM over z = 0 is the identity and conserves energy;
- the Fresnel LCT (free space) agrees with the ASM to the paraxial error
  wherever the chirp is sampled (dx * span <= lambda z).
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O


def test_abcd_elements_and_composition():
    from dlux_gb300.layers import abcd_propagators as ap
    els = [ap.ABCDFreeSpace(1.0), ap.ABCDLens(2.0), ap.ABCDMirror(3.0), ap.ABCDConjugatePlane(4.0)]
    refs = [O.abcd_free_space(1.0), O.abcd_lens(2.0), O.abcd_mirror(3.0), O.abcd_fraunhofer(4.0)]
    for el, ref in zip(els, refs):
        assert isinstance(el.abcd, torch.Tensor) and el.abcd.shape == (2, 2)
        np.testing.assert_allclose(el.abcd.numpy(), ref)
    # elements apply in order: free space then lens is lens @ free
    m = ap.compose_abcd([els[0].abcd, els[1].abcd]).numpy()
    np.testing.assert_allclose(m, O.abcd_lens(2.0) @ O.abcd_free_space(1.0))
    np.testing.assert_allclose(m, O.compose_abcd([O.abcd_free_space(1.0), O.abcd_lens(2.0)]))
    # every ray-transfer matrix here has unit determinant
    for ref in refs:
        assert abs(np.linalg.det(ref) - 1.0) < 1e-12


def test_abcd_propagator_base_and_getattr():
    from dlux_gb300.coordinates import CoordSpec
    from dlux_gb300.layers import abcd_propagators as ap
    spec = CoordSpec(n=8, d=1 / 32, c=0.0)
    prop = ap.MFTPropagator([ap.ABCDFreeSpace(1.0), ap.ABCDLens(2.0)], spec)
    assert prop.n == 8
    assert isinstance(prop.ABCDFreeSpace, ap.ABCDFreeSpace)
    assert np.allclose(prop.focal_length, 2.0)
    assert prop.abcd.shape == (2, 2)
    with pytest.raises(AttributeError):
        prop.not_an_attr


def test_constructor_errors():
    from dlux_gb300.coordinates import CoordSpec
    from dlux_gb300.layers import abcd_propagators as ap
    with pytest.raises(ValueError, match="can not specify d"):
        ap.FFTPropagator([ap.ABCDFreeSpace(1.0)], CoordSpec(n=8, d=1.0, c=0.0))
    with pytest.raises(ValueError, match="can not specify d or c"):
        ap.ASMPropagator(1.0, CoordSpec(n=8, d=1.0, c=0.0))
    prop = ap.ASMPropagator(1.0, CoordSpec(n=8, c=None))
    assert prop.distance.shape == ()
    assert prop.n == 8
    with pytest.raises(AttributeError):
        prop.not_an_attr
    with pytest.raises(TypeError):
        ap.Fraunhofer()
    with pytest.raises(TypeError):
        ap.Fresnel()
    for cls in (ap.Fraunhofer, ap.Fresnel):
        concrete = type("Concrete", (cls,), {"__call__": lambda self, w: w})
        with pytest.raises(NotImplementedError):
            concrete()
    # B = 0 (imaging condition) has no Collins integral
    with pytest.raises(ValueError, match="B = 0"):
        ap.lct_axes(ap.abcd_lens(1.0), [1e-6], 8, 0.1, 0.0, 8, 0.1, 0.0)
    with pytest.raises(ValueError, match="afocal"):
        ap.abcd_effective_focal_length(ap.abcd_free_space(1.0))


def test_oracle_fraunhofer_lct_is_the_mft():
    n, m, wl, f = 32, 24, 1e-6, 2.0
    dx, dout = 1.0 / n, 2.5e-6
    rng = np.random.default_rng(0)
    u = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    L = O.lct_direct(u, O.coord_xs(n, dx), O.coord_xs(m, dout), wl, O.abcd_fraunhofer(f))
    M = O.mft(u, wl, dx, m, dout, focal_length=f)
    assert np.linalg.norm(L - (-1j * dx / dout) * M) / np.linalg.norm(L) < 1e-12


def test_oracle_asm_identity_and_energy():
    rng = np.random.default_rng(1)
    n, dx, wl = 32, 1e-5, 1e-6
    u = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    a = O.asm_prop(u, dx, wl, 0.0, 40)
    lo = (40 - n) // 2
    np.testing.assert_allclose(a[lo:lo + n, lo:lo + n], u, atol=1e-12)
    assert np.abs(a).sum() - np.abs(a[lo:lo + n, lo:lo + n]).sum() < 1e-10
    # propagating components only (dx >> lambda): |H| = 1, energy is conserved
    b = O.asm_prop(u, dx, wl, 0.3, 64)
    assert abs((np.abs(b) ** 2).sum() / (np.abs(u) ** 2).sum() - 1.0) < 1e-12


@pytest.mark.parametrize("n,dx,z,w", [(64, 20e-6, 0.2, 120e-6), (128, 10e-6, 0.1, 100e-6)])
def test_oracle_fresnel_lct_matches_asm(n, dx, z, w):
    wl, P = 1e-6, 256
    xs = O.coord_xs(n, dx)
    X, Y = np.meshgrid(xs, xs)
    g = np.exp(-(X ** 2 + Y ** 2) / (2 * w ** 2)).astype(complex)
    A = O.asm_prop(g, dx, wl, z, P) * np.exp(-2j * np.pi * ((z / wl) % 1.0))
    L = O.lct_direct(g, xs, O.coord_xs(P, dx), wl, O.abcd_free_space(z))
    assert np.linalg.norm(L - A) / np.linalg.norm(A) < 1e-5
