"""GPU parity of the fused polychromatic PSF and its hand-written gradient.

Errors are relative L2 norms against the FP64 oracle. Tolerances: PSF <= 1e-5
for both arithmetic forms; gradients <= 1e-5 in both forms (the reported values in the test output are
typically far lower).
"""

import os

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
VARIANTS = ["fp32", "split_bf16"]


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_case(n, m, nz, L, seed, spiders=False):
    rng = np.random.default_rng(seed)
    kw = dict(secondary_diameter=0.1)
    if spiders:
        kw.update(spider_width=0.01, spider_angles=(0, 90, 180, 270))
    T, B = O.circular_aperture(n, 1.0, oversample=3, zernike_nolls=list(range(4, 4 + nz)), **kw)
    c = rng.normal(0, 40e-9, nz)
    wls = np.linspace(0.8e-6, 1.2e-6, L)
    w = rng.dirichlet(np.ones(L))
    return T, B, c, wls, w


def to_dev(x, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("n,m,L", [(64, 32, 3), (128, 256, 4), (256, 128, 2)])
def test_poly_psf_matches_oracle(cuda, variant, n, m, L):
    from dlux_gb300 import kernels
    T, B, c, wls, w = make_case(n, m, 10, L, 7)
    opd = O.eval_basis(B, c)
    ps_out = float(O.arcsec2rad(0.02 / 2))
    ref = O.poly_psf(T, opd, wls, w, 1.0, m, ps_out)
    plan = kernels.PolyPlan(wls, n, 1.0 / n, m, ps_out, variant=variant)
    amp = to_dev(T)
    scale = kernels.amp_norm(amp)
    got = plan.psf(amp, scale, to_dev(opd), None, to_dev(w)).cpu().numpy()
    err = rel(got, ref)
    print(f"poly psf {variant} n={n} m={m} L={L}: rel L2 {err:.2e}")
    assert err < 1e-5


@pytest.mark.parametrize("variant", VARIANTS)
def test_poly_psf_grad_matches_oracle(cuda, variant):
    from dlux_gb300 import kernels
    n, m, L = 128, 64, 3
    T, B, c, wls, w = make_case(n, m, 10, L, 11)
    rng = np.random.default_rng(12)
    opd = O.eval_basis(B, c)
    phase = rng.normal(0, 0.1, (n, n)) * (T > 0)
    tilt = (0.05e-6, -0.03e-6)
    ps_out = float(O.arcsec2rad(0.02))
    G = rng.normal(size=(m, m))
    Teff = T / np.sqrt((T ** 2).sum())
    ref = O.poly_psf_grad(Teff, opd, wls, w, 1.0, m, ps_out, G, phase=phase, offset=tilt)
    plan = kernels.PolyPlan(wls, n, 1.0 / n, m, ps_out, variant=variant)
    amp = to_dev(T)
    scale = kernels.amp_norm(amp)
    gr = plan.grad(amp, scale, to_dev(opd), to_dev(phase), to_dev(w), to_dev(G), tilt)
    errs = {k: rel(gr[{"g_amp": "amp", "g_opd": "opd", "g_phase": "phase", "g_w": "w"}[k]]
                   .cpu().numpy(), ref[k]) for k in ref}
    print(f"poly grad {variant}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    for k, v in errs.items():
        assert v < 1e-5, (k, v)


@pytest.mark.parametrize("variant", VARIANTS)
def test_poly_psf_golden_fixture(cuda, variant):
    """Committed FP64 fixture (tests/golden/make_golden.py)."""
    from dlux_gb300 import kernels
    g = np.load(os.path.join(HERE, "golden", "poly_small.npz"))
    plan = kernels.PolyPlan(g["wavelengths"], int(g["n"]), float(g["pixel_scale_in"]),
                            int(g["m"]), float(g["pixel_scale_out"]), variant=variant)
    amp = to_dev(g["transmission"])
    scale = kernels.amp_norm(amp)
    psf = plan.psf(amp, scale, to_dev(g["opd"]), None, to_dev(g["weights"])).cpu().numpy()
    assert rel(psf, g["psf"]) < 1e-5
    gr = plan.grad(amp, scale, to_dev(g["opd"]), None, to_dev(g["weights"]), to_dev(g["g_psf"]))
    assert rel(gr["opd"].cpu().numpy(), g["g_opd"]) < 1e-5


def test_split_form_meets_1e5_at_config2_size(cuda):
    """512 pupil -> 512 focal, 8 of the 64 wavelengths: PSF and gradient error vs FP64."""
    from dlux_gb300 import kernels
    n, m, L = 512, 512, 8
    T, B, c, wls, w = make_case(n, m, 21, L, 2, spiders=True)
    opd = O.eval_basis(B, c)
    ps_out = float(O.arcsec2rad(0.02 / 4))
    ref = O.poly_psf(T, opd, wls, w, 1.0, m, ps_out)
    plan = kernels.PolyPlan(wls, n, 1.0 / n, m, ps_out, variant="split_bf16")
    amp = to_dev(T)
    scale = kernels.amp_norm(amp)
    got = plan.psf(amp, scale, to_dev(opd), None, to_dev(w)).cpu().numpy()
    err = rel(got, ref)
    rng = np.random.default_rng(3)
    G = rng.normal(size=(m, m))
    Teff = T / np.sqrt((T ** 2).sum())
    gref = O.poly_psf_grad(Teff, opd, wls, w, 1.0, m, ps_out, G)
    gr = plan.grad(amp, scale, to_dev(opd), None, to_dev(w), to_dev(G), want=("opd",))
    gerr = rel(gr["opd"].cpu().numpy(), gref["g_opd"])
    print(f"config-2 size split_bf16: psf rel L2 {err:.2e}, g_opd rel L2 {gerr:.2e}")
    assert err < 1e-5
    assert gerr < 1e-5


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("n,m", [(128, 64), (128, 96)])
def test_kept_focal_fields_give_the_same_gradient(cuda, variant, n, m):
    """A forward that keeps its focal fields F lets the reusing backward form
    F-bar = 2 G F elementwise instead of repeating the y-contraction GEMM. Both
    backwards match the FP64 oracle (relative L2 <= 1e-5) and each other:
    within 1e-6 in the FP32 form (rounding order), within 3e-6 in the split
    form, where F-bar's hi/lo split quantises the two paths' (equally accurate)
    values differently. A backward whose inputs differ from the kept forward's
    recomputes everything (bitwise equal to a backward without reuse).

    The cotangent has mean 1 (as a likelihood's typically has): with a
    zero-mean one, the wavelength-weight gradient <G, |F_l|^2> / w_l is a sum
    over the focal plane that cancels to a small fraction of its terms, and
    its relative error grows by that ratio in either backward."""
    from dlux_gb300 import kernels
    L = 3
    T, B, c, wls, w = make_case(n, m, 10, L, 11)
    rng = np.random.default_rng(12)
    opd = O.eval_basis(B, c)
    phase = rng.normal(0, 0.1, (n, n)) * (T > 0)
    tilt = (0.04e-6, -0.02e-6)
    ps_out = float(O.arcsec2rad(0.02))
    G = 1.0 + 0.5 * rng.normal(size=(m, m))
    Teff = T / np.sqrt((T ** 2).sum())
    ref = O.poly_psf_grad(Teff, opd, wls, w, 1.0, m, ps_out, G, phase=phase, offset=tilt)
    plan = kernels.PolyPlan(wls, n, 1.0 / n, m, ps_out, variant=variant)
    amp = to_dev(T)
    scale = kernels.amp_norm(amp)
    args = (amp, scale, to_dev(opd), to_dev(phase), to_dev(w))
    keys = {"amp": "g_amp", "opd": "g_opd", "phase": "g_phase", "w": "g_w"}
    out = {}
    for keep in (False, True):
        p0 = plan.psf(*args, tilt=tilt, keep=keep).clone()
        tok = plan.forward_token()
        assert tok != 0
        gr = plan.grad(*args, to_dev(G), tilt, reuse_token=tok)
        out[keep] = (p0.cpu().numpy(), {k: v.cpu().numpy() for k, v in gr.items()})
    assert np.array_equal(out[False][0], out[True][0])   # the PSF is the same launch
    tol_same = 1e-6 if variant == "fp32" else 3e-6
    for k, kr in keys.items():
        e_same = rel(out[True][1][k], out[False][1][k])
        e_keep = rel(out[True][1][k], ref[kr])
        e_recompute = rel(out[False][1][k], ref[kr])
        print(f"kept focal fields {variant} {n}->{m} {k}: vs recompute {e_same:.2e}, "
              f"vs oracle {e_keep:.2e} (recomputing backward {e_recompute:.2e})")
        assert e_same < tol_same and e_keep < 1e-5 and e_recompute < 1e-5
    # kept fields of another forward are not used
    opd2 = to_dev(opd * 1.1)
    args2 = (amp, scale, opd2, to_dev(phase), to_dev(w))
    plan.psf(*args, tilt=tilt, keep=True)
    tok = plan.forward_token()
    g_reuse = plan.grad(*args2, to_dev(G), tilt, reuse_token=tok)
    g_fresh = plan.grad(*args2, to_dev(G), tilt)
    for k in keys:
        assert torch.equal(g_reuse[k], g_fresh[k]), k
    plan.close()
