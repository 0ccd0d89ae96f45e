"""Forward-to-backward reuse of the poly plan's workspace.

A backward that starts from the forward's pupil field and first-stage product
(dlx_poly_reuse_forward) runs the same kernels on the same values as one that
recomputes them, so the gradients must agree bit for bit. A token is refused,
and the backward recomputes, when another call used the plan in between or the
inputs differ.
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu


def dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device="cuda")


def setup(variant, seed=0, n=128, m=64, L=4):
    from dlux_gb300 import kernels
    rng = np.random.default_rng(seed)
    T, B = O.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 12)))
    wls = np.linspace(0.9e-6, 1.1e-6, L)
    ps = float(O.arcsec2rad(0.03))
    plan = kernels.PolyPlan(wls, n, 1 / n, m, ps, variant=variant)
    amp = dev(T)
    inputs = []
    for k in range(2):
        opd = dev(O.eval_basis(B, rng.normal(0, 50e-9, B.shape[0])))
        inputs.append(dict(amp=amp, amp_scale=kernels.amp_norm(amp), opd=opd, phase=None,
                           weights=dev(rng.dirichlet(np.ones(L)))))
    G = dev(rng.normal(size=(m, m)))
    return plan, inputs, G


def grads(plan, x, G, token=0):
    g = plan.grad(x["amp"], x["amp_scale"], x["opd"], x["phase"], x["weights"], G,
                  want=("amp", "opd", "w"), reuse_token=token)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in g.items() if v is not None}


def psf(plan, x):
    return plan.psf(x["amp"], x["amp_scale"], x["opd"], x["phase"], x["weights"])


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_reuse_is_bitwise_equal_to_recompute(cuda, variant):
    plan, (a, _), G = setup(variant)
    ref = grads(plan, a, G)                 # recomputes (no forward before it)
    psf(plan, a)
    tok = plan.forward_token()
    assert tok != 0
    got = grads(plan, a, G, token=tok)      # starts from the forward's workspace
    assert plan.forward_token() == 0        # the reverse pass consumed the state
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_stale_or_foreign_token_recomputes(cuda, variant):
    plan, (a, b), G = setup(variant, seed=1)
    ref_a = grads(plan, a, G)
    # another forward in between: the token of a's forward is stale
    psf(plan, a)
    tok_a = plan.forward_token()
    psf(plan, b)
    assert plan.forward_token() not in (0, tok_a)
    got = grads(plan, a, G, token=tok_a)
    for k in ref_a:
        np.testing.assert_array_equal(got[k], ref_a[k], err_msg=k)
    # the forward state of b with the inputs of a: refused by the input check
    psf(plan, b)
    got = grads(plan, a, G, token=plan.forward_token())
    for k in ref_a:
        np.testing.assert_array_equal(got[k], ref_a[k], err_msg=k)
    # a request covers one backward only
    psf(plan, a)
    tok = plan.forward_token()
    g1 = grads(plan, a, G, token=tok)
    g2 = grads(plan, a, G, token=tok)
    for k in ref_a:
        np.testing.assert_array_equal(g1[k], ref_a[k], err_msg=k)
        np.testing.assert_array_equal(g2[k], ref_a[k], err_msg=k)


def test_autograd_step_uses_reuse_and_matches_oracle(cuda):
    """The PolyPSF autograd path (forward, then backward with the forward's
    token) against the FP64 oracle gradient."""
    import dlux_gb300 as dl
    rng = np.random.default_rng(3)
    n, m = 128, 64
    T, B = O.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 14)))
    c = rng.normal(0, 50e-9, 10)
    wls = [0.9e-6, 1.0e-6, 1.1e-6]
    coeffs = torch.as_tensor(c, dtype=torch.float32, device="cuda").requires_grad_(True)
    optics = dl.AngularOpticalSystem(
        n, 1.0, [dl.TransmissiveLayer(dev(T), normalise=True), dl.BasisLayer(dev(B), coeffs)],
        m, 0.02)
    R = rng.normal(size=(m, m))
    (optics.propagate(wls) * dev(R)).sum().backward()
    torch.cuda.synchronize()
    opd = O.eval_basis(B, c)
    ps = float(O.arcsec2rad(0.02))
    Teff = T / np.sqrt((T ** 2).sum())
    w = np.full(len(wls), 1.0 / len(wls))
    g = O.poly_psf_grad(Teff, opd, wls, w, 1.0, m, ps, R)
    gc = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))
    err = np.linalg.norm(coeffs.grad.cpu().numpy() - gc) / np.linalg.norm(gc)
    assert err < 1e-5
