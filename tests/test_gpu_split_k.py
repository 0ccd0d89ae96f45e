"""Split K for GEMMs that leave most SMs idle (small pupils, few wavelengths).

A poly plan of the config-1 shape (256^2 pupil -> 128^2 PSF, one wavelength)
splits every GEMM. The tests check that:
- the split path runs (one reduction launch per split GEMM);
- PSF and gradients agree with a plan made with split K off and with the
  FP64 oracle, within the split form's 1e-5.
Objects alone vs in a batch of one plan (bitwise) are covered by
test_gpu_batched.py, whose small shapes split K.
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


def make(split, max_objects=1, n=256, m=128, wls=(1e-6,)):
    from dlux_gb300 import _lib, kernels
    lib = _lib.load()
    _lib.check(lib.dlx_set_split_k(1 if split else 0))
    try:
        return kernels.PolyPlan(list(wls), n, 1.0 / n, m, float(O.arcsec2rad(0.02)),
                                variant="split_bf16", max_objects=max_objects)
    finally:
        _lib.check(lib.dlx_set_split_k(1))


def inputs(n=256, m=128, L=1, seed=0):
    from dlux_gb300 import kernels
    rng = np.random.default_rng(seed)
    T, B = O.circular_aperture(n, 1.0, oversample=1, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 14)))
    amp = dev(T)
    opd = O.eval_basis(B, rng.normal(0, 50e-9, B.shape[0]))
    return dict(T=T, opd=opd, amp=amp, amp_scale=kernels.amp_norm(amp), opd_d=dev(opd),
                w=dev(np.full(L, 1.0 / L)), G=dev(rng.normal(size=(m, m))))


def run(plan, x):
    from dlux_gb300 import _lib
    lib = _lib.load()
    lib.dlx_launch_count.restype = ctypes.c_longlong
    torch.cuda.synchronize()
    c0 = lib.dlx_launch_count()
    psf = plan.psf(x["amp"], x["amp_scale"], x["opd_d"], None, x["w"])
    g = plan.grad(x["amp"], x["amp_scale"], x["opd_d"], None, x["w"], x["G"],
                  want=("opd", "amp"))
    torch.cuda.synchronize()
    return psf.cpu().numpy(), g["opd"].cpu().numpy(), g["amp"].cpu().numpy(), \
        lib.dlx_launch_count() - c0


def test_split_k_runs_and_matches_unsplit_and_oracle(cuda):
    x = inputs()
    on, off = make(True), make(False)
    psf1, go1, ga1, n1 = run(on, x)
    psf0, go0, ga0, n0 = run(off, x)
    assert n1 > n0, (n1, n0)  # the reductions of the split GEMMs
    assert rel(psf1, psf0) < 1e-5
    assert rel(go1, go0) < 1e-5 and rel(ga1, ga0) < 1e-5
    ps = float(O.arcsec2rad(0.02))
    Teff = x["T"] / np.sqrt((x["T"] ** 2).sum())
    ref = O.poly_psf(Teff, x["opd"], [1e-6], [1.0], 1.0, 128, ps)
    assert rel(psf1, ref) < 1e-5
    g = O.poly_psf_grad(Teff, x["opd"], [1e-6], [1.0], 1.0, 128, ps, x["G"].cpu().numpy())
    assert rel(go1, g["g_opd"]) < 1e-5
