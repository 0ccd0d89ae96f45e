"""Paired form of the tensor-core GEMM (two-CTA clusters, cta_group::2 MMAs;
opt-in, off by default).

The paired and single-CTA forms compute every output element from the same
products in the same K order, so poly-plan PSFs and gradients must be
bitwise equal with the pairing switched on and off. Shapes:
- the benchmark's 512^2 -> 512^2 (four 128-column tiles: every GEMM pairs);
- ragged 200^2 -> 240^2 (a partial second tile, a partial last K block, and
  M not a multiple of 128);
- 256^2 -> 384^2 (three tiles: the focal GEMMs stay single-CTA).
Each run also checks the device status word (no timed-out wait) and the
FP64 oracle.
"""

import ctypes

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu


def dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device="cuda")


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def set_pair(on):
    from dlux_gb300 import _lib
    _lib.check(_lib.load().dlx_set_gemm_pair(1 if on else 0))


def case(n, m, L, seed):
    from dlux_gb300 import kernels
    rng = np.random.default_rng(seed)
    T, B = O.circular_aperture(n, 1.0, oversample=1, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 12)))
    opd = O.eval_basis(B, rng.normal(0, 40e-9, B.shape[0]))
    wls = np.linspace(0.9e-6, 1.1e-6, L)
    w = rng.dirichlet(np.ones(L))
    amp = dev(T)
    return dict(T=T, opd=opd, wls=wls, w=w, amp=amp, amp_scale=kernels.amp_norm(amp),
                opd_d=dev(opd), w_d=dev(w), G=rng.normal(size=(m, m)))


def run(plan, x):
    from dlux_gb300 import _lib
    G = dev(x["G"])
    psf = plan.psf(x["amp"], x["amp_scale"], x["opd_d"], None, x["w_d"])
    g = plan.grad(x["amp"], x["amp_scale"], x["opd_d"], None, x["w_d"], G, want=("opd", "amp"))
    torch.cuda.synchronize()
    assert _lib.device_status() == 0
    return psf.cpu().numpy(), g["opd"].cpu().numpy(), g["amp"].cpu().numpy()


def test_pair_form_is_available(cuda):
    from dlux_gb300 import _lib
    n = ctypes.c_int(0)
    _lib.check(_lib.load().dlx_gemm_pair_clusters(ctypes.byref(n)))
    print(f"co-resident two-CTA clusters: {n.value}")
    assert n.value >= 1


@pytest.mark.parametrize("n,m,L", [(512, 512, 8), (200, 240, 3), (256, 384, 2)])
def test_pair_matches_single_cta_and_oracle(cuda, n, m, L):
    from dlux_gb300 import kernels
    x = case(n, m, L, seed=n + m)
    ps = float(O.arcsec2rad(0.02))
    from dlux_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.dlx_set_split_k(0))  # split-K GEMMs never pair: keep every GEMM whole
    try:
        plan = kernels.PolyPlan(list(x["wls"]), n, 1.0 / n, m, ps, variant="split_bf16")
    finally:
        _lib.check(lib.dlx_set_split_k(1))
    try:
        set_pair(True)
        psf1, go1, ga1 = run(plan, x)
        set_pair(False)
        psf0, go0, ga0 = run(plan, x)
    finally:
        set_pair(False)  # the default
        plan.close()
    e = (rel(psf1, psf0), rel(go1, go0), rel(ga1, ga0))
    same = bool(np.array_equal(psf1, psf0) and np.array_equal(go1, go0))
    print(f"{n}->{m} x {L}: paired vs single-CTA rel {e}, bitwise equal: {same}")
    assert same and max(e) == 0.0
    Teff = x["T"] / np.sqrt((x["T"] ** 2).sum())
    ref = O.poly_psf(Teff, x["opd"], x["wls"], x["w"], 1.0, m, ps)
    assert rel(psf1, ref) < 1e-5
    g = O.poly_psf_grad(Teff, x["opd"], x["wls"], x["w"], 1.0, m, ps, x["G"])
    assert rel(go1, g["g_opd"]) < 1e-5


def test_per_plan_gemm_form_is_bitwise_the_global_one(cuda):
    """dlx_poly_plan_set_gemm_form (the autotuner's per-plan launch form): a plan made
    with gemm_pair=True gives the bits of the global switch's paired form, one with
    gemm_pair=False those of the single-CTA form, whatever the global switch says; a plan
    with split_k=False keeps every GEMM whole and still matches the oracle."""
    from dlux_gb300 import kernels
    n, m, L = 256, 256, 4
    x = case(n, m, L, 21)
    ps = float(O.arcsec2rad(0.02))
    clusters = ctypes.c_int(0)
    from dlux_gb300 import _lib
    _lib.check(_lib.load().dlx_gemm_pair_clusters(ctypes.byref(clusters)))
    if clusters.value == 0:
        pytest.skip("paired form unavailable")
    try:
        set_pair(True)
        ref_pair = run(kernels.PolyPlan(x["wls"], n, 1.0 / n, m, ps, variant="split_bf16"), x)
        set_pair(False)
        ref_single = run(kernels.PolyPlan(x["wls"], n, 1.0 / n, m, ps, variant="split_bf16"), x)
        # per-plan forms against the opposite global setting
        on = run(kernels.PolyPlan(x["wls"], n, 1.0 / n, m, ps, variant="split_bf16",
                                  gemm_pair=True), x)
        set_pair(True)
        off = run(kernels.PolyPlan(x["wls"], n, 1.0 / n, m, ps, variant="split_bf16",
                                   gemm_pair=False), x)
    finally:
        set_pair(False)
    for a, b in zip(on, ref_pair):
        assert np.array_equal(a, b)
    for a, b in zip(off, ref_single):
        assert np.array_equal(a, b)
    whole = run(kernels.PolyPlan(x["wls"], n, 1.0 / n, m, ps, variant="split_bf16",
                                 split_k=False), x)
    ref = O.poly_psf(x["T"], x["opd"], x["wls"], x["w"], 1.0, m, ps)
    assert rel(whole[0], ref) < 1e-5
