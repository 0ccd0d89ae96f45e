"""torch.autograd.Function wrappers over the C ABI.

Each Function's forward and backward call the library's kernels; the
backward passes are the hand-written adjoints. The polychromatic PSF's
forward keeps its focal fields in the plan's workspace when a gradient is
needed, and its backward starts from them when nothing used the plan in
between (otherwise it recomputes them).
"""

from __future__ import annotations

import torch

from . import kernels


class BasisEval(torch.autograd.Function):
    """opd = base + sum_k c_k B_k (dLux utils/math.py:177-196)."""

    @staticmethod
    def forward(ctx, basis, coeffs, base):
        ctx.save_for_backward(basis)
        ctx.coeff_shape = tuple(coeffs.shape)
        ctx.has_base = base is not None
        return kernels.basis_eval(basis.detach(), coeffs.detach(),
                                  None if base is None else base.detach().contiguous())

    @staticmethod
    def backward(ctx, g):
        (basis,) = ctx.saved_tensors
        g = g.contiguous()
        g_c = kernels.basis_grad(basis, g, ctx.coeff_shape) if ctx.needs_input_grad[1] else None
        g_base = g if (ctx.has_base and ctx.needs_input_grad[2]) else None
        return None, g_c, g_base


def eval_basis(basis, coeffs, base=None):
    return BasisEval.apply(basis, coeffs, base)


class PolyPSF(torch.autograd.Function):
    """sum_l |MFT_l(sqrt(w_l) A exp(i (2 pi (opd + tilt)/lambda_l + phase)))|^2.

    A = amp * sqrt(1 / sum amp^2) when ``normalise`` (TransmissiveLayer with
    normalise=True, wavefronts.py:397-424), else amp. amp/opd/phase may be None.
    """

    @staticmethod
    def forward(ctx, plan, normalise, amp, opd, phase, weights, tilt, amp_scale=None):
        # amp_scale: the normalisation of amp, when the caller computed it already
        if not (normalise and amp is not None):
            amp_scale = None
        elif amp_scale is None:
            amp_scale = kernels.amp_norm(amp.detach())
        t = (float(tilt[0]), float(tilt[1]))
        ctx.plan, ctx.normalise, ctx.tilt = plan, normalise, t
        ctx.tilt_device = tilt.device
        ctx.save_for_backward(amp, opd, phase, weights, amp_scale)
        # with a reverse pass ahead, the forward keeps its focal fields as well
        keep = any(ctx.needs_input_grad[2:7])
        psf = plan.psf(_d(amp), amp_scale, _d(opd), _d(phase), weights.detach().contiguous(), t,
                       keep=keep)
        # the backward may start from this forward's workspace if nothing used the plan since
        ctx.token = plan.forward_token()
        return psf

    @staticmethod
    def backward(ctx, g_psf):
        amp, opd, phase, weights, amp_scale = ctx.saved_tensors
        plan = ctx.plan
        want = []
        if ctx.needs_input_grad[2] and amp is not None:
            want.append("amp")
        if (ctx.needs_input_grad[3] and opd is not None) or ctx.needs_input_grad[6]:
            want.append("opd")
        if ctx.needs_input_grad[4] and phase is not None:
            want.append("phase")
        if ctx.needs_input_grad[5]:
            want.append("w")
        if not want:
            return (None,) * 8
        gr = plan.grad(_d(amp), amp_scale, _d(opd), _d(phase), weights.detach().contiguous(),
                       g_psf.contiguous(), ctx.tilt, tuple(want), reuse_token=ctx.token)
        g_amp = gr["amp"]
        if g_amp is not None and ctx.normalise:
            g_amp = kernels.amp_norm_backward(amp.detach(), g_amp)
        g_tilt = None
        if ctx.needs_input_grad[6]:
            # d/d(theta_x, theta_y) of opd + theta_x X + theta_y Y: project on the pixel grid
            g_tilt = kernels.basis_grad(plan.tilt_basis(), gr["opd"], (2,)).to(
                device=ctx.tilt_device, dtype=torch.float64)
        g_opd = gr["opd"] if (ctx.needs_input_grad[3] and opd is not None) else None
        return None, None, g_amp, g_opd, gr["phase"], gr["w"], g_tilt, None


def _d(t):
    return None if t is None else t.detach().contiguous()


def poly_psf(plan, amp, opd, phase, weights, normalise=False, tilt=None, amp_scale=None):
    """Fused polychromatic PSF; ``tilt`` is a float64 tensor [2] (radians), may require grad.
    ``amp_scale``: sqrt(1 / sum amp^2) computed by the caller (else here, when normalising)."""
    if tilt is None:
        tilt = torch.zeros(2, dtype=torch.float64)
    tilt = torch.as_tensor(tilt, dtype=torch.float64)
    return PolyPSF.apply(plan, bool(normalise), amp, opd, phase, weights, tilt, amp_scale)


class PolySources(torch.autograd.Function):
    """Summed PSF of many point sources sharing one pupil (sources.py:392-411).

    Each source is an object of a batched plan: its own tilt (position) and
    spectral weights (spectrum x flux); the DFT operands of every wavelength
    are shared, so one launch covers wavelengths x sources.
    """

    @staticmethod
    def forward(ctx, plan, normalise, base_tilt, amp, opd, phase, weights, positions):
        amp_scale = kernels.amp_norm(amp.detach()) if (normalise and amp is not None) else None
        w = weights.detach().contiguous()
        pos = positions.detach().to(torch.float64).cpu()
        tilts = [(float(pos[s, 0]) + base_tilt[0], float(pos[s, 1]) + base_tilt[1])
                 for s in range(pos.shape[0])]
        ctx.plan, ctx.normalise, ctx.tilts = plan, normalise, tilts
        ctx.pos_device = positions.device
        ctx.save_for_backward(amp, opd, phase, weights, amp_scale)
        out = torch.empty((plan.n_out, plan.n_out), dtype=torch.float32, device=w.device)
        objs = [dict(amp=_d(amp), amp_scale=amp_scale, opd=_d(opd), phase=_d(phase), weights=w[s],
                     tilt=tilts[s]) for s in range(len(tilts))]
        plan.forward_objects(objs, psf_sum=out)
        return out

    @staticmethod
    def backward(ctx, g):
        amp, opd, phase, weights, amp_scale = ctx.saved_tensors
        plan = ctx.plan
        S = len(ctx.tilts)
        n, dev = plan.n_in, g.device
        g = g.contiguous()
        want_amp = ctx.needs_input_grad[3] and amp is not None
        want_opd = ctx.needs_input_grad[4] and opd is not None
        want_ph = ctx.needs_input_grad[5] and phase is not None
        g_amp = torch.empty((n, n), device=dev) if want_amp else None
        g_opd = torch.empty((n, n), device=dev) if want_opd else None
        g_ph = torch.empty((n, n), device=dev) if want_ph else None
        g_w = torch.empty_like(weights, dtype=torch.float32) if ctx.needs_input_grad[6] else None
        g_t = torch.empty((S, 2), device=dev) if ctx.needs_input_grad[7] else None
        w = weights.detach().contiguous()
        objs = [dict(amp=_d(amp), amp_scale=amp_scale, opd=_d(opd), phase=_d(phase), weights=w[s],
                     tilt=ctx.tilts[s], g_psf=g, g_w=None if g_w is None else g_w[s],
                     g_tilt=None if g_t is None else g_t[s]) for s in range(S)]
        plan.backward_objects(objs, sum_grads={"amp": g_amp, "opd": g_opd, "phase": g_ph})
        if g_amp is not None and ctx.normalise:
            g_amp = kernels.amp_norm_backward(amp.detach(), g_amp)
        g_pos = None if g_t is None else g_t.to(device=ctx.pos_device, dtype=torch.float64)
        return None, None, None, g_amp, g_opd, g_ph, g_w, g_pos


def poly_sources(plan, amp, opd, phase, weights, positions, normalise=False, base_tilt=(0.0, 0.0)):
    """Summed PSF of sources at ``positions`` [S, 2] (radians) with weights [S, L]."""
    return PolySources.apply(plan, bool(normalise), (float(base_tilt[0]), float(base_tilt[1])),
                             amp, opd, phase, weights, positions)


class ScenePSF(torch.autograd.Function):
    """Summed image of many point sources through one pupil (sources.py:392-411),
    differentiable w.r.t. the source positions and the per-(source, wavelength)
    weights. The pupil (amplitude, OPD, phase) is a constant here; the tilt of
    each source is an output-coordinate shift of its DFT matrices."""

    @staticmethod
    def forward(ctx, plan, amp, amp_scale, opd, phase, weights, positions, base_tilt):
        pos = positions.detach().to(device="cuda", dtype=torch.float64)
        if base_tilt[0] != 0.0 or base_tilt[1] != 0.0:
            pos = pos + torch.tensor(base_tilt, dtype=torch.float64, device=pos.device)
        w = weights.detach().to(torch.float32).contiguous()
        ctx.plan, ctx.pos_device = plan, positions.device
        ctx.save_for_backward(amp, amp_scale, opd, phase, w, pos)
        out = plan.forward(_d(amp), amp_scale, _d(opd), _d(phase), pos, w)
        ctx.token = plan.forward_token()  # retained fields, if the plan kept them
        return out

    @staticmethod
    def backward(ctx, g):
        amp, amp_scale, opd, phase, w, pos = ctx.saved_tensors
        want_w = ctx.needs_input_grad[5]
        want_pos = ctx.needs_input_grad[6]
        if not (want_w or want_pos):
            return None, None, None, None, None, None, None, None
        g_pos, g_w = ctx.plan.backward(_d(amp), amp_scale, _d(opd), _d(phase), pos, w,
                                       g.contiguous(), want_pos, want_w, reuse_token=ctx.token)
        if g_pos is not None:
            g_pos = g_pos.to(device=ctx.pos_device, dtype=torch.float64)
        return None, None, None, None, None, g_w, g_pos, None


def scene_psf(plan, amp, opd, phase, weights, positions, normalise=False,
              base_tilt=(0.0, 0.0)):
    """Summed image of sources at ``positions`` [S, 2] (rad) with weights [S, L]."""
    amp_scale = kernels.amp_norm(amp.detach()) if (normalise and amp is not None) else None
    return ScenePSF.apply(plan, amp, amp_scale, opd, phase, weights, positions,
                          (float(base_tilt[0]), float(base_tilt[1])))


class DynamicZernike(torch.autograd.Function):
    """OPD = sum_j c_j Z_j of a dynamic aperture, evaluated per pixel on the device
    (polynomials.py:20-51); the reverse pass recomputes the Zernikes per pixel."""

    @staticmethod
    def forward(ctx, desc, noll, coeffs):
        ctx.desc, ctx.noll = desc, list(noll)
        _, opd = kernels.aberrated_aperture(desc, noll, coeffs.detach(), want_trans=False)
        return opd

    @staticmethod
    def backward(ctx, g):
        if not ctx.needs_input_grad[2]:
            return None, None, None
        return None, None, kernels.aberrated_aperture_grad(ctx.desc, ctx.noll, g.contiguous())


def dynamic_zernike(desc, noll, coeffs):
    return DynamicZernike.apply(desc, list(noll), coeffs)


class Conv2dSame(torch.autograd.Function):
    """jax.scipy.signal.convolve(x, kernel, mode="same") with both gradients."""

    @staticmethod
    def forward(ctx, x, kernel):
        ctx.save_for_backward(x, kernel)
        return kernels.conv2d_same(x.detach().to(torch.float32), kernel.detach())

    @staticmethod
    def backward(ctx, g):
        x, kernel = ctx.saved_tensors
        gx, gk = kernels.conv2d_same_backward(x.detach().to(torch.float32), kernel.detach(),
                                              g.contiguous(), ctx.needs_input_grad[0],
                                              ctx.needs_input_grad[1])
        if gk is not None:
            gk = gk.to(kernel.dtype)
        return gx, gk


def conv2d_same(x, kernel):
    if not isinstance(kernel, torch.Tensor):
        kernel = torch.as_tensor(kernel, dtype=torch.float32, device=x.device)
    return Conv2dSame.apply(x, kernel.to(device=x.device))


class LinearTransform(torch.autograd.Function):
    """A cached MFT or FFT plan applied to complex64 fields; backward is the adjoint."""

    @staticmethod
    def forward(ctx, plan, field):
        ctx.plan = plan
        return plan.forward(field.detach())

    @staticmethod
    def backward(ctx, g):
        return None, ctx.plan.adjoint(g.contiguous())


def apply_plan(plan, field):
    return LinearTransform.apply(plan, field)


class DownsampleFlat(torch.autograd.Function):
    """k x k block sum times a pixel response (array_ops.py:124-162, detector_layers.py:100-131)."""

    @staticmethod
    def forward(ctx, psf, flat, k, mean):
        ctx.k, ctx.mean = k, mean
        ctx.save_for_backward(psf, flat)
        return kernels.downsample(psf.detach().contiguous(), k, mean,
                                  None if flat is None else flat.detach().contiguous())

    @staticmethod
    def backward(ctx, g):
        psf, flat = ctx.saved_tensors
        want_flat = flat is not None and ctx.needs_input_grad[1]
        g_in, g_flat = kernels.downsample_backward(
            psf.detach().contiguous(), g.contiguous(), ctx.k, ctx.mean,
            None if flat is None else flat.detach().contiguous(), want_flat)
        return (g_in if ctx.needs_input_grad[0] else None), g_flat, None, None


def downsample(psf, k, mean=False, flat=None):
    return DownsampleFlat.apply(psf, flat, int(k), bool(mean))


class PhasorMul(torch.autograd.Function):
    """field * amp * exp(i (2 pi opd / lambda_b + phase)) for a batch of wavelengths.

    The forward runs the phasor kernel, the backward its hand-written reverse
    kernel (dlx_phasor_backward), which rebuilds the phasors with the forward's
    own error-free reduction. Used by the layer-by-layer path; the fused system
    path has its own reverse kernels.
    """

    @staticmethod
    def forward(ctx, wavelengths, pixel_scale, field, amp, opd, phase):
        n = field.shape[-1]
        out = kernels.phasor(wavelengths, n, pixel_scale, field=field.detach().contiguous(),
                             amp=_d(amp), opd=_d(opd), phase=_d(phase))
        ctx.wavelengths = wavelengths
        ctx.save_for_backward(field, amp, opd, phase)
        return out

    @staticmethod
    def backward(ctx, g):
        field, amp, opd, phase = ctx.saved_tensors
        need = ctx.needs_input_grad
        g_field, g_amp, g_opd, g_phase = kernels.phasor_backward(
            ctx.wavelengths, field.detach().contiguous(), _d(amp), _d(opd), _d(phase), g,
            want_field=need[2], want_amp=amp is not None and need[3],
            want_opd=opd is not None and need[4], want_phase=phase is not None and need[5])
        return None, None, g_field, g_amp, g_opd, g_phase


class PsfSum(torch.autograd.Function):
    """PSF = sum_b w_b |F_b|^2 of unweighted focal fields (optical_systems.py:211-223):
    the weighted intensity kernel and its reverse kernel."""

    @staticmethod
    def forward(ctx, field, weights):
        f = field.detach().contiguous()
        w = None if weights is None else weights.detach()
        ctx.save_for_backward(f, w)
        return kernels.psf_sum_weighted(f, w)

    @staticmethod
    def backward(ctx, g):
        f, w = ctx.saved_tensors
        gf, gw = kernels.psf_sum_weighted_backward(
            f, w, g, want_field=ctx.needs_input_grad[0],
            want_weights=w is not None and ctx.needs_input_grad[1])
        if gw is not None:
            gw = gw.to(w.dtype)
        return gf, gw


def psf_sum(field, weights=None):
    return PsfSum.apply(field, weights)


class Normalise(torch.autograd.Function):
    """Wavefront.normalise (wavefronts.py:397-424) per plane, with its reverse kernel."""

    @staticmethod
    def forward(ctx, field, mode, value):
        f = field.detach().contiguous()
        ctx.save_for_backward(f)
        ctx.mode, ctx.value = mode, value
        return kernels.normalise(f, mode, value)

    @staticmethod
    def backward(ctx, g):
        (f,) = ctx.saved_tensors
        return kernels.normalise_backward(f, g, ctx.mode, ctx.value), None, None


def normalise(field, mode="power", value=1.0):
    return Normalise.apply(field, mode, float(value))
