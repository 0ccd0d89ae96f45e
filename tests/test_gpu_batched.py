"""Batched objects of the fused plan: every object's result is the same alone and in a batch.

Objects (serving requests, point sources) share the per-wavelength DFT
operands and run as one set of launches. Each object's tiles and reductions
use exactly the arithmetic of a one-object plan, so results are compared
bit for bit; the oracle check uses the tolerances of the other PSF tests.
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


def objects(n, L, R, seed):
    rng = np.random.default_rng(seed)
    T, B = O.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 12)))
    out = []
    for r in range(R):
        T_r = T * (1 + 0.01 * rng.normal(size=T.shape))
        opd = O.eval_basis(B, rng.normal(0, 50e-9, B.shape[0]))
        w = rng.dirichlet(np.ones(L)) * rng.uniform(0.5, 2.0)
        tilt = rng.normal(0, 2e-7, 2)
        out.append(dict(T=T_r, opd=opd, w=w, tilt=tuple(tilt)))
    return out


def dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device="cuda")


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_objects_alone_equal_objects_in_batch(cuda, variant):
    from dlux_gb300 import kernels
    n, m, L, R = 128, 64, 3, 5
    wls = np.linspace(0.9e-6, 1.1e-6, L)
    ps = float(O.arcsec2rad(0.03))
    objs = objects(n, L, R, 1)
    batched = kernels.PolyPlan(wls, n, 1 / n, m, ps, variant=variant, max_objects=4)
    single = kernels.PolyPlan(wls, n, 1 / n, m, ps, variant=variant, max_objects=1)
    rng = np.random.default_rng(2)
    Gs = [dev(rng.normal(size=(m, m))) for _ in range(R)]
    descs, singles = [], []
    for o, G in zip(objs, Gs):
        amp = dev(o["T"])
        d = dict(amp=amp, amp_scale=kernels.amp_norm(amp), opd=dev(o["opd"]), weights=dev(o["w"]),
                 tilt=o["tilt"], psf=torch.empty((m, m), device="cuda"), g_psf=G,
                 g_opd=torch.empty((n, n), device="cuda"), g_amp=torch.empty((n, n), device="cuda"),
                 g_w=torch.empty(L, device="cuda"), g_tilt=torch.empty(2, device="cuda"))
        descs.append(d)
        s = {k: (v.clone() if isinstance(v, torch.Tensor) and k.startswith(("psf", "g_"))
                 and k != "g_psf" else v) for k, v in d.items()}
        singles.append(s)
    total = torch.empty((m, m), device="cuda")
    batched.forward_objects(descs, psf_sum=total)       # 5 objects: chunks of 4 and 1
    batched.backward_objects(descs)
    for s in singles:
        single.forward_objects([s])
        single.backward_objects([s])
    torch.cuda.synchronize()
    for d, s in zip(descs, singles):
        for k in ("psf", "g_opd", "g_amp", "g_w", "g_tilt"):
            assert torch.equal(d[k], s[k]), k
    assert torch.allclose(total, sum(d["psf"] for d in descs), rtol=1e-6, atol=0)
    # oracle check of two objects
    for o, d in list(zip(objs, descs))[:2]:
        ref = O.poly_psf(o["T"], o["opd"], wls, o["w"], 1.0, m, ps, offset=o["tilt"])
        assert rel(d["psf"].cpu().numpy(), ref) < 1e-5


def test_summed_pixel_gradients(cuda):
    from dlux_gb300 import kernels
    n, m, L, R = 64, 32, 2, 3
    wls = [1.0e-6, 1.1e-6]
    ps = float(O.arcsec2rad(0.05))
    objs = objects(n, L, R, 3)
    plan = kernels.PolyPlan(wls, n, 1 / n, m, ps, variant="fp32", max_objects=2)
    amp = dev(objs[0]["T"])
    scale = kernels.amp_norm(amp)
    opd = dev(objs[0]["opd"])
    G = dev(np.random.default_rng(4).normal(size=(m, m)))
    descs = [dict(amp=amp, amp_scale=scale, opd=opd, weights=dev(o["w"]), tilt=o["tilt"],
                  g_psf=G, g_opd=torch.empty((n, n), device="cuda")) for o in objs]
    plan.backward_objects(descs)
    per = sum(d["g_opd"] for d in descs)
    summed = torch.empty((n, n), device="cuda")
    plan.backward_objects([{k: v for k, v in d.items() if k != "g_opd"} for d in descs],
                          sum_grads={"opd": summed})
    assert torch.allclose(summed, per, rtol=1e-5, atol=1e-6 * per.abs().max().item())


def test_point_sources_flux_and_position_gradients(cuda):
    """Many-source scene through PointSources.model (batched plan), vs FP64 differences."""
    import dlux_gb300 as dl
    rng = np.random.default_rng(5)
    n, m = 64, 32
    T, B = O.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 10)))
    c = rng.normal(0, 40e-9, B.shape[0])
    wls = np.array([0.9e-6, 1.1e-6])
    S = 6
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
        tot = 0.0
        for (x, y), fl in zip(p, f):
            tot += (G * O.poly_psf(T, opd, wls, [0.5 * fl, 0.5 * fl], 1.0, m, ps,
                                   offset=(x, y))).sum()
        return tot
    p0, f0 = pos.detach().numpy(), flux.detach().cpu().numpy().astype(float)
    ref_img = sum(O.poly_psf(T, opd, wls, [0.5 * fl, 0.5 * fl], 1.0, m, ps, offset=tuple(p))
                  for p, fl in zip(p0, f0))
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


def test_shared_plan_workspace_and_generated_operand(cuda):
    """A plan without its own buffers, run on an attached workspace, gives the same bits
    as a plan that owns them; the generated-operand form matches the oracle."""
    from dlux_gb300 import kernels
    n, m, L = 128, 64, 3
    o = objects(n, L, 1, 21)[0]
    wls = np.linspace(0.8e-6, 1.2e-6, L)
    ps = float(O.arcsec2rad(0.01))
    amp = dev(o["T"])
    scale = kernels.amp_norm(amp)
    args = (amp, scale, dev(o["opd"]), None, dev(o["w"]))
    # shared-workspace plans do not split K; compare with an owning plan that does not either
    from dlux_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.dlx_set_split_k(0))
    try:
        own = kernels.PolyPlan(wls, n, 1.0 / n, m, ps, variant="split_bf16", max_objects=2)
    finally:
        _lib.check(lib.dlx_set_split_k(1))
    shared = kernels.PolyPlan(wls, n, 1.0 / n, m, ps, variant="split_bf16", max_objects=2,
                              own_workspace=False)
    assert shared.footprint < own.footprint
    with pytest.raises(Exception):
        shared.psf(*args)                      # no workspace attached yet
    nbytes = shared.workspace_bytes()
    buf = torch.empty(nbytes + 256, dtype=torch.uint8, device="cuda")
    off = (-buf.data_ptr()) % 256
    with pytest.raises(ValueError):
        shared.attach_workspace(buf[off:off + nbytes - 256])    # too small
    shared.attach_workspace(buf[off:off + nbytes])
    a = own.psf(*args).cpu().numpy()
    b = shared.psf(*args).cpu().numpy()
    assert np.array_equal(a, b)
    gen = kernels.PolyPlan(wls, n, 1.0 / n, m, ps, variant="split_bf16", operand_mode=1)
    c = gen.psf(*args).cpu().numpy()
    ref = O.poly_psf(o["T"], o["opd"], wls, o["w"], 1.0, m, ps)
    print(f"generated-operand psf: rel L2 {rel(c, ref):.2e}; loaded {rel(a, ref):.2e}")
    assert rel(c, ref) < 1e-5
    with pytest.raises(ValueError):
        kernels.PolyPlan(wls, n, 1.0 / n, m, ps, variant="split_bf16", operand_mode=7)


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_forward_backward_matches_separate_passes(cuda, variant):
    """The one-sweep PSF + reverse pass (cotangent known up front) gives the same bits as
    the forward pass followed by the recomputing reverse pass."""
    from dlux_gb300 import kernels
    n, m, L, R = 128, 64, 3, 3
    objs_np = objects(n, L, R, 31)
    wls = np.linspace(0.8e-6, 1.2e-6, L)
    ps = float(O.arcsec2rad(0.01))
    plan = kernels.PolyPlan(wls, n, 1.0 / n, m, ps, variant=variant, max_objects=R)
    rng = np.random.default_rng(32)

    def make():
        out = []
        for o in objs_np:
            amp = dev(o["T"])
            out.append(dict(amp=amp, amp_scale=kernels.amp_norm(amp), opd=dev(o["opd"]),
                            weights=dev(o["w"]), tilt=o["tilt"],
                            g_psf=dev(rng.normal(size=(m, m))),
                            psf=torch.empty((m, m), device="cuda"),
                            g_opd=torch.empty((n, n), device="cuda"),
                            g_amp=torch.empty((n, n), device="cuda"),
                            g_w=torch.empty((L,), device="cuda"),
                            g_tilt=torch.empty((2,), device="cuda")))
        return out
    a = make()
    rng = np.random.default_rng(32)
    b = make()
    plan.forward_objects(a)
    plan.backward_objects(a)
    plan.forward_backward_objects(b)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        for k in ("psf", "g_opd", "g_amp", "g_w", "g_tilt"):
            assert torch.equal(x[k], y[k]), f"{k} differs between the two reverse paths"
