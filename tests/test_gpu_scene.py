"""Many point sources through one pupil (scene plan): the tilt of each source as a shift
of its DFT output coordinates. Checked against the FP64 oracle (image), against the
per-source-field path (image and gradients), and by FP64 central differences (positions,
weights). Tolerances: image relative L2 <= 1e-5; gradients <= 1e-5 against the
per-source path and against the oracle's fourth-order central differences (position step
2e-9 rad).
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def dev(x, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def scene(n, m, L, S, seed, span=0.3):
    rng = np.random.default_rng(seed)
    T, B = O.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 12)))
    opd = O.eval_basis(B, rng.normal(0, 40e-9, B.shape[0]))
    wls = np.linspace(0.8e-6, 1.2e-6, L)
    pos = rng.uniform(-span, span, (S, 2)) * np.pi / 180 / 3600
    w = rng.uniform(0.2, 2.0, (S, L))
    return T, opd, wls, pos, w


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
@pytest.mark.parametrize("n,m,L,S", [(64, 32, 2, 5), (256, 64, 3, 40), (100, 36, 2, 9),
                                     (90, 45, 2, 6)])
def test_scene_image_matches_oracle_and_per_source_path(cuda, variant, n, m, L, S):
    """Sides 100 / 36 and 90 / 45 are not multiples of 8: split rows padded (the
    tilted-matrix kernel's four-element path at 100, its scalar path at 90)."""
    from dlux_gb300 import kernels
    T, opd, wls, pos, w = scene(n, m, L, S, 3)
    ps = float(O.arcsec2rad(0.02))
    amp = dev(T)
    scale = kernels.amp_norm(amp)
    plan = kernels.ScenePlan(wls, n, 1.0 / n, m, ps, variant=variant, max_sources=32)
    img = plan.forward(amp, scale, dev(opd), None, torch.as_tensor(pos), dev(w)).cpu().numpy()
    ref = sum(O.poly_psf(T, opd, wls, w[s], 1.0, m, ps, offset=tuple(pos[s])) for s in range(S))
    err = rel(img, ref)
    print(f"scene {variant} n={n} m={m} L={L} S={S}: image rel L2 {err:.2e}")
    assert err < 1e-5
    # the per-source-field path on the same inputs, image and gradients
    pplan = kernels.PolyPlan(wls, n, 1.0 / n, m, ps, variant=variant, max_objects=min(S, 32))
    G = dev(np.random.default_rng(4).normal(size=(m, m)))
    g_pos, g_w = plan.backward(amp, scale, dev(opd), None, torch.as_tensor(pos), dev(w), G)
    gt = torch.empty((S, 2), device="cuda")
    gw = torch.empty((S, L), device="cuda")
    objs = [dict(amp=amp, amp_scale=scale, opd=dev(opd), weights=dev(w[s]), tilt=tuple(pos[s]),
                 g_psf=G, g_tilt=gt[s], g_w=gw[s]) for s in range(S)]
    pplan.backward_objects(objs, sum_grads={})
    e_pos, e_w = rel(g_pos.cpu(), gt.cpu()), rel(g_w.cpu(), gw.cpu())
    print(f"  vs per-source path: positions {e_pos:.2e}, weights {e_w:.2e}")
    assert e_pos < 1e-5 and e_w < 1e-5


def test_point_sources_scene_gradients_vs_differences(cuda):
    """PointSources.model routes a fixed pupil through the scene plan; flux and position
    gradients against FP64 central differences of the oracle."""
    import dlux_gb300 as dl
    rng = np.random.default_rng(8)
    n, m = 64, 32
    T, B = O.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 10)))
    c = rng.normal(0, 40e-9, B.shape[0])
    wls = np.array([0.9e-6, 1.1e-6])
    S = 5
    pos = torch.tensor(rng.uniform(-0.1, 0.1, (S, 2)) * np.pi / 180 / 3600, dtype=torch.float64,
                       requires_grad=True)
    flux = torch.tensor(10 ** rng.uniform(0, 2, S), dtype=torch.float32, device="cuda",
                        requires_grad=True)
    optics = dl.AngularOpticalSystem(n, 1.0, [dl.TransmissiveLayer(dev(T), normalise=True),
                                              dl.BasisLayer(dev(B), dev(c))], m, 0.04)
    img = dl.PointSources(wls, position=pos, flux=flux).model(optics)
    G = rng.normal(size=(m, m))
    (img * dev(G)).sum().backward()
    opd = O.eval_basis(B, c)
    ps = float(O.arcsec2rad(0.04))

    def loss(p, f):
        return sum((G * O.poly_psf(T, opd, wls, [0.5 * fl, 0.5 * fl], 1.0, m, ps,
                                   offset=tuple(q))).sum() for q, fl in zip(p, f))
    p0, f0 = pos.detach().numpy(), flux.detach().cpu().numpy().astype(float)
    ref_img = sum(O.poly_psf(T, opd, wls, [0.5 * fl, 0.5 * fl], 1.0, m, ps, offset=tuple(q))
                  for q, fl in zip(p0, f0))
    assert rel(img.detach().cpu().numpy(), ref_img) < 1e-5
    gf = np.array([(loss(p0, f0 + 1e-3 * np.eye(S)[s]) - loss(p0, f0 - 1e-3 * np.eye(S)[s]))
                   / 2e-3 for s in range(S)])
    assert rel(flux.grad.cpu().numpy(), gf) < 1e-5
    # fourth-order central differences in FP64 (step 2e-9 rad: truncation ~1e-9)
    h = 2e-9
    gp = np.zeros_like(p0)
    for s in range(S):
        for k in range(2):
            d = np.zeros_like(p0)
            d[s, k] = h
            gp[s, k] = (-loss(p0 + 2 * d, f0) + 8 * loss(p0 + d, f0) - 8 * loss(p0 - d, f0)
                        + loss(p0 - 2 * d, f0)) / (12 * h)
    assert rel(pos.grad.numpy(), gp) < 1e-5


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_retained_fields_give_the_recomputed_bits(cuda, variant):
    """A backward that starts from the forward's retained D1 / Y.D1 (several
    source chunks) gives the same image and gradients, bit for bit, as one
    that recomputes them; a stale token or a different input falls back to
    the recomputation."""
    from dlux_gb300 import kernels
    n, m, L, S = 128, 64, 3, 40
    T, opd, wls, pos, w = scene(n, m, L, S, 9)
    ps = float(O.arcsec2rad(0.02))
    amp = dev(T)
    scale = kernels.amp_norm(amp)
    opd_d, pos_t, w_d = dev(opd), dev(pos, torch.float64), dev(w)
    G = dev(np.random.default_rng(5).normal(size=(m, m)))
    plan = kernels.ScenePlan(wls, n, 1.0 / n, m, ps, variant=variant, max_sources=16)

    # reference: no retention
    plan.set_retain_limit(0)
    img0 = plan.forward(amp, scale, opd_d, None, pos_t, w_d).clone()
    assert plan.forward_token() == 0
    gp0, gw0 = plan.backward(amp, scale, opd_d, None, pos_t, w_d, G)
    # retained: 3 chunks of at most 16 sources
    plan.set_retain_limit(1 << 34)
    img1 = plan.forward(amp, scale, opd_d, None, pos_t, w_d).clone()
    tok = plan.forward_token()
    assert tok != 0
    gp1, gw1 = plan.backward(amp, scale, opd_d, None, pos_t, w_d, G, reuse_token=tok)
    torch.cuda.synchronize()
    assert torch.equal(img0, img1)
    assert torch.equal(gp0, gp1) and torch.equal(gw0, gw1)
    # a second backward may reuse the same retained state
    gp2, gw2 = plan.backward(amp, scale, opd_d, None, pos_t, w_d, G, reuse_token=tok)
    assert torch.equal(gp0, gp2) and torch.equal(gw0, gw2)
    # stale token: another forward (other weights) replaced the retained state
    w2 = dev(w * 1.5)
    plan.forward(amp, scale, opd_d, None, pos_t, w2)
    gp3, gw3 = plan.backward(amp, scale, opd_d, None, pos_t, w_d, G, reuse_token=tok)
    assert torch.equal(gp0, gp3) and torch.equal(gw0, gw3)
    # current token but different inputs (weights pointer): recomputed
    gp4, gw4 = plan.backward(amp, scale, opd_d, None, pos_t, w_d, G,
                             reuse_token=plan.forward_token())
    assert torch.equal(gp0, gp4) and torch.equal(gw0, gw4)
