"""Generates tests/golden/*.npz from the FP64 oracle (run: python tests/golden/make_golden.py).

The reference (dLux on JAX) cannot be imported in this environment, so the
fixtures are produced by the NumPy FP64 restatement in ``oracle/`` after it has
been checked against the reference's own known-answer tests
(tests/test_oracle.py). Inputs are seeded PCG64 draws.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import dlux_oracle as O  # noqa: E402


def poly_small():
    rng = np.random.default_rng(20261203)
    n, m, L = 64, 32, 3
    T, B = O.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 14)))
    c = rng.normal(0, 50e-9, B.shape[0])
    opd = O.eval_basis(B, c)
    wls = np.linspace(0.9e-6, 1.1e-6, L)
    w = rng.dirichlet(np.ones(L))
    ps_out = float(O.arcsec2rad(0.04))
    psf = O.poly_psf(T, opd, wls, w, 1.0, m, ps_out)
    G = rng.normal(size=(m, m))
    Teff = T / np.sqrt((T ** 2).sum())
    g = O.poly_psf_grad(Teff, opd, wls, w, 1.0, m, ps_out, G)
    np.savez_compressed(os.path.join(HERE, "poly_small.npz"), n=n, m=m,
                        pixel_scale_in=1.0 / n, pixel_scale_out=ps_out, wavelengths=wls,
                        weights=w, transmission=T.astype(np.float32), opd=opd.astype(np.float32),
                        coefficients=c, basis=B.astype(np.float32), psf=psf, g_psf=G,
                        g_opd=g["g_opd"], g_amp=g["g_amp"], g_w=g["g_w"])


def mft_small():
    rng = np.random.default_rng(7)
    E = (rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))) / 32
    cases = {}
    for i, (fl, inv, pix) in enumerate([(2.0, False, True), (None, True, False),
                                        (2.0, True, False), (None, False, True)]):
        cases[f"out_{i}"] = O.mft(E, 1.0, 0.1, 16, 0.05, fl, (1.0, -2.0), pix, inv)
    np.savez_compressed(os.path.join(HERE, "mft_small.npz"), field=E, **cases)


if __name__ == "__main__":
    poly_small()
    mft_small()
    print("written")
