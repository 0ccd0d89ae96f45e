"""PSF convolution (mode "same") on the device: PSF.convolve, ApplyJitter, ResolvedSource,
PointResolvedSource against the FP64 oracle, with gradients. Tolerances: relative L2 <= 1e-5
for values and gradients (FP32 sums of at most a few thousand products). Batches of images
share one kernel: its gradient is the sum over the batch. A kernel nearly as tall as the
image leaves some row bands of the kernel-gradient reduction without valid rows."""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device="cuda")


@pytest.mark.parametrize("Bt,H,W,K0,K1", [(1, 64, 64, 3, 3), (1, 100, 70, 8, 5),
                                          (1, 128, 128, 33, 33), (1, 40, 40, 1, 7),
                                          (3, 64, 48, 5, 7), (3, 40, 40, 33, 9),
                                          (2, 16, 20, 15, 3)])
def test_conv_same_and_gradients(cuda, Bt, H, W, K0, K1):
    from dlux_gb300 import autograd
    rng = np.random.default_rng(H + K0 + 100 * Bt)
    a = rng.random((Bt, H, W))
    k = rng.random((K0, K1))
    G = rng.normal(size=(Bt, H, W))
    x = dev(a if Bt > 1 else a[0]).requires_grad_(True)
    kt = dev(k).requires_grad_(True)
    out = autograd.conv2d_same(x, kt)
    (out * dev(G if Bt > 1 else G[0])).sum().backward()
    ref = np.stack([O.convolve_same(a[b], k) for b in range(Bt)])
    # <conv(a, k), G> is linear in k: d/dk[i][j] = sum_b <conv(a_b, e_ij), G_b>
    g_k = np.array([[sum((O.convolve_same(a[b], np.eye(1, K0 * K1, i * K1 + j)
                                           .reshape(K0, K1)) * G[b]).sum() for b in range(Bt))
                     for j in range(K1)] for i in range(K0)])
    # and in a: d/da_b is the correlation of G_b with k
    g_a = np.zeros_like(a)
    s0, s1 = (K0 - 1) // 2, (K1 - 1) // 2
    for b in range(Bt):
        Gp = np.pad(G[b], ((K0, K0), (K1, K1)))
        for p in range(K0):
            for q in range(K1):
                g_a[b] += k[p, q] * Gp[K0 - s0 + p:K0 - s0 + p + H, K1 - s1 + q:K1 - s1 + q + W]
    out_np = out.detach().cpu().numpy().reshape(Bt, H, W)
    ga_np = x.grad.cpu().numpy().reshape(Bt, H, W)
    e_o, e_a, e_k = rel(out_np, ref), rel(ga_np, g_a), rel(kt.grad.cpu(), g_k)
    print(f"conv {Bt}x{H}x{W} * {K0}x{K1}: out {e_o:.2e}, d/din {e_a:.2e}, d/dk {e_k:.2e}")
    assert e_o < 1e-5 and e_a < 1e-5 and e_k < 1e-5


def test_jitter_and_resolved_sources(cuda):
    import dlux_gb300 as dl
    rng = np.random.default_rng(3)
    n, m = 64, 32
    T, B = O.circular_aperture(n, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 10)))
    c = rng.normal(0, 40e-9, B.shape[0])
    wls = np.array([0.9e-6, 1.1e-6])
    optics = dl.AngularOpticalSystem(n, 1.0, [dl.TransmissiveLayer(dev(T), normalise=True),
                                              dl.BasisLayer(dev(B), dev(c))], m, 0.04)
    ps = float(O.arcsec2rad(0.04))
    opd = O.eval_basis(B, c)
    pos = (2e-7, -1e-7)
    base = O.poly_psf(T, opd, wls, [0.5, 0.5], 1.0, m, ps, offset=pos)
    # jitter
    jit = dl.ApplyJitter(1.3)
    kj = O.jitter_kernel(1.3)
    assert rel(jit.kernel.cpu(), kj) < 1e-6
    psf = dl.PointSource(wls, position=pos).model(optics, return_psf=True)
    out = dl.LayeredDetector([jit]).model(psf)
    assert rel(out.detach().cpu(), O.convolve_same(base, kj)) < 1e-5
    # resolved source, gradient w.r.t. the distribution
    dist = rng.random((5, 5))
    d = dev(dist).requires_grad_(True)
    src = dl.ResolvedSource(wls, position=pos, flux=2.0, distribution=d)
    img = src.model(optics)
    G = rng.normal(size=(m, m))
    (img * dev(G)).sum().backward()
    dn = dist / dist.sum()
    ref = O.convolve_same(2.0 * base, dn)
    assert rel(img.detach().cpu(), ref) < 1e-5
    # d/d dist through the normalisation: finite differences of the oracle
    def loss(dd):
        return (O.convolve_same(2.0 * base, dd / dd.sum()) * G).sum()
    # (fourth-order central differences in FP64: accurate to ~1e-10 here)
    gd = np.zeros_like(dist)
    h = 1e-4
    for i in range(5):
        for j in range(5):
            e = np.zeros_like(dist)
            e[i, j] = h
            gd[i, j] = (-loss(dist + 2 * e) + 8 * loss(dist + e) - 8 * loss(dist - e)
                        + loss(dist - 2 * e)) / (12 * h)
    assert rel(d.grad.cpu(), gd) < 1e-5
    # point + resolved with a contrast
    prs = dl.PointResolvedSource(wls, position=pos, flux=3.0, distribution=dist, contrast=0.5)
    img2 = prs.model(optics)
    fp, fr = 2 * 0.5 * 3.0 / 1.5, 2 * 3.0 / 1.5
    ref2 = fp * base + O.convolve_same(fr * base, dn)
    assert rel(img2.detach().cpu(), ref2) < 1e-5
    with pytest.raises(NotImplementedError):
        prs.model(optics, return_wf=True)
