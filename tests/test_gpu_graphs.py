"""A whole PSF + gradient step replayed as one CUDA graph gives the eager step's bits."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_graphed_step_matches_eager(cuda):
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    from dlux_gb300.graphs import GraphedStep

    rng = np.random.default_rng(7)
    T, B = dlu.circular_aperture(128, 1.0, oversample=1, secondary_diameter=0.1,
                                 zernike_nolls=list(range(4, 14)))
    c0 = torch.as_tensor(rng.normal(0, 50e-9, 10), dtype=torch.float32, device="cuda")
    R = torch.as_tensor(rng.normal(size=(64, 64)), dtype=torch.float32, device="cuda")
    optics = dl.AngularOpticalSystem(128, 1.0, [dl.TransmissiveLayer(T, normalise=True),
                                                dl.BasisLayer(B, c0)], 64, 0.04, 1)

    def step(c_in):
        c = c_in.detach().requires_grad_(True)
        psf = optics.set("layers.BasisLayer.coefficients", c).propagate([1e-6, 1.2e-6])
        loss = (psf * R).sum()
        loss.backward()
        return loss.detach(), c.grad

    g = GraphedStep(step, c0)
    for seed in (1, 2):
        c = torch.as_tensor(np.random.default_rng(seed).normal(0, 50e-9, 10),
                            dtype=torch.float32, device="cuda")
        loss_g, grad_g = (t.clone() for t in g(c))
        loss_e, grad_e = step(c)
        torch.cuda.synchronize()
        assert torch.equal(loss_g, loss_e)
        assert torch.equal(grad_g, grad_e)
    with pytest.raises(ValueError):
        g(torch.zeros(3, device="cuda"))


def test_graphed_phase_retrieval_step_matches_eager(cuda):
    """The phase-retrieval step (amplitude, coefficient and flat-field
    gradients of a Poisson NLL through a detector) replayed as one CUDA graph
    gives the eager step's bits, for new coefficients each replay."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    from dlux_gb300.graphs import GraphedStep

    rng = np.random.default_rng(8)
    T, B = dlu.circular_aperture(128, 1.0, oversample=1, secondary_diameter=0.1,
                                 zernike_nolls=list(range(4, 16)))
    f32 = dict(dtype=torch.float32, device="cuda")
    A0 = torch.as_tensor(np.asarray(T.cpu() if hasattr(T, "cpu") else T)
                         * (1 + rng.normal(0, 0.01, (128, 128))), **f32)
    c0 = torch.as_tensor(rng.normal(0, 40e-9, 12), **f32)
    flat0 = torch.as_tensor(1 + rng.normal(0, 0.02, (64, 64)), **f32)
    data = torch.as_tensor(rng.poisson(1e3, (64, 64)).astype(np.float32), **f32)
    wls = [0.95e-6, 1.05e-6]
    optics = dl.AngularOpticalSystem(128, 1.0, [dl.TransmissiveLayer(A0, normalise=True),
                                                dl.BasisLayer(B, c0)], 64, 0.04, 1)

    def step(c_in):
        A = A0.detach().requires_grad_(True)
        c = c_in.detach().requires_grad_(True)
        flat = flat0.detach().requires_grad_(True)
        sys_ = optics.set(["layers.TransmissiveLayer.transmission",
                           "layers.BasisLayer.coefficients"], [A, c])
        img = dl.LayeredDetector([dl.ApplyPixelResponse(flat)]).model(
            sys_.propagate(wls, return_psf=True)) * 1e6
        loss = (img - data * torch.log(img)).sum()
        loss.backward()
        return loss.detach(), c.grad, A.grad, flat.grad

    g = GraphedStep(step, c0)
    for k in range(3):
        c = c0 * (1.0 + 0.1 * k)
        got = [t.clone() for t in g(c)]
        ref = step(c)
        torch.cuda.synchronize()
        for a, b in zip(got, ref):
            assert torch.equal(a, b)


def test_graphed_step_host_io_matches_device_graph(cuda):
    """GraphedStep(host_io=True) holds the host copies inside the graph: host
    coefficients in, pinned host outputs back, the same bits as the device-mode
    graph for new coefficients each call."""
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    from dlux_gb300.graphs import GraphedStep

    rng = np.random.default_rng(9)
    T, B = dlu.circular_aperture(128, 1.0, oversample=1, secondary_diameter=0.1,
                                 zernike_nolls=list(range(4, 14)))
    c0 = torch.as_tensor(rng.normal(0, 50e-9, 10), dtype=torch.float32, device="cuda")
    R = torch.as_tensor(rng.normal(size=(64, 64)), dtype=torch.float32, device="cuda")
    optics = dl.AngularOpticalSystem(128, 1.0, [dl.TransmissiveLayer(T, normalise=True),
                                                dl.BasisLayer(B, c0)], 64, 0.04, 1)

    def step(c_in):
        c = c_in.detach().requires_grad_(True)
        psf = optics.set("layers.BasisLayer.coefficients", c).propagate([1e-6, 1.2e-6])
        loss = (psf * R).sum()
        loss.backward()
        return loss.detach(), c.grad, None

    g = GraphedStep(step, c0)
    gh = GraphedStep(step, c0.cpu(), host_io=True)
    for seed in (3, 4):
        c = torch.as_tensor(np.random.default_rng(seed).normal(0, 50e-9, 10),
                            dtype=torch.float32)
        loss_d, grad_d, _ = g(c.cuda())
        loss_d, grad_d = loss_d.cpu(), grad_d.cpu()
        loss_h, grad_h, none_h = gh(c)
        assert not loss_h.is_cuda and loss_h.is_pinned() and none_h is None
        assert torch.equal(loss_h, loss_d) and torch.equal(grad_h, grad_d)
