"""Benchmark: PSF+gradient evaluations per second on one GB300.

Workload (the polychromatic split-precision configuration): 512 x 512 pupil
of a 1 m circular aperture with a 10 cm central obscuration and four 1 cm
spider vanes, 21 Noll Zernikes (j = 4..24) with N(0, 30 nm) coefficients,
64 wavelengths uniform on 0.8-1.2 um with Dirichlet(1) weights, MFT to
512 x 512 at 4x oversampling of a 0.02"/px detector, then a 4 x 4 sum
downsample to 128 x 128. One step = one PSF evaluation plus the gradient of
sum(R * image) (R a seeded N(0, 1) 128 x 128 array) with respect to the 21
coefficients, through the public API (AngularOpticalSystem.propagate,
LayeredDetector, torch autograd -> the hand-written reverse kernels). The step
is captured once as a CUDA graph (dlux_gb300.graphs.GraphedStep, the counterpart
of jax.jit of the step) and replayed: `value` times the replays with the inputs
resident, `e2e` adds the pinned host copies every step. The eager step is also
timed (`eager_value`); it gives the per-launch GEMM times of the roofline.

Every step touches ~1 GB of device memory (cached DFT matrices plus the
per-wavelength fields), far more than the 129 MB L2, so no explicit L2 flush
is made between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--variant split_bf16|fp32]
  python bench.py --impl reference   # the CPU restatement of the same step
  python bench.py --workload serving # mixed-shape request stream through the server
  python bench.py --workload cfg1|cfg3|cfg4   # the other measured configurations
  python bench.py --workload fft     # FFT propagation: radix line FFTs vs DFT-GEMM forms
"""

from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N_PUPIL = 512
N_FOCAL = 512
OVERSAMPLE = 4
PSF_PIXEL_SCALE = 0.02  # arcsec per detector pixel
N_WAVELENGTHS = 64
NOLLS = list(range(4, 25))
SEED = 2
METRIC = "PSF+grad evals/sec"
# Individually timed steps for the p50/p99 latencies (outside the K-step timed region).
LATENCY_SAMPLES = 200
# Whole steps of the CPU restatement timed for the GPU line's cpu_baseline.
CPU_BASELINE_STEPS = 3
# DRAM bytes (read + write) of one tensor-core GEMM launch per wavelength, from an ncu
# capture of the four GEMM launches of a 16-wavelength step of this workload (71.2 MB
# per launch on average, / 16). Traffic grows in proportion to the wavelength count
# (each wavelength is an independent GEMM on its own operands).
GEMM_DRAM_BYTES_PER_WAVELENGTH = 71.2e6 / 16


def config_dict(extra=None):
    d = {"workload": "polychromatic PSF + coefficient gradient: 512^2 pupil (D=1 m, 10% "
                     "obscuration, 4 x 1 cm spiders), 21 Zernikes N(0,30nm), 64 lambda "
                     "0.8-1.2 um Dirichlet(1), MFT 512^2 at 4x oversampling, 4x4 sum "
                     "downsample to 128^2, grad of sum(R*image) w.r.t. coefficients",
         "pupil": N_PUPIL, "focal": N_FOCAL, "wavelengths": N_WAVELENGTHS,
         "zernikes": len(NOLLS), "detector": 128,
         "l2": "inputs larger than L2 (~1 GB of device state touched per step), no flush"}
    if extra:
        d.update(extra)
    return d


def make_inputs(seed=SEED):
    """Seeded synthetic inputs (NumPy PCG64), shared by every implementation."""
    rng = np.random.default_rng(seed)
    coeffs = rng.normal(0, 30e-9, len(NOLLS))
    wls = np.linspace(0.8e-6, 1.2e-6, N_WAVELENGTHS)
    weights = rng.dirichlet(np.ones(N_WAVELENGTHS))
    R = rng.normal(size=(128, 128))
    return coeffs, wls, weights, R


# ----------------------------------------------------------------------------
# Clock sampling during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------
# CPU arm: the oracle's complex64 restatement of dLux's op order
# ----------------------------------------------------------------------------
_CPU = {}


def _cpu_worker_init(T, Teff, ps_out):
    _CPU.update(T=T, Teff=Teff, ps_out=ps_out)


def _cpu_worker(job):
    """PSF and opd-gradient partial sums of one block of wavelengths (complex64 port)."""
    from oracle import dlux_oracle as O
    opd, wls, weights, G = job
    psf = O.poly_psf(_CPU["T"], opd, wls, weights, 1.0, N_FOCAL, _CPU["ps_out"],
                     precision="c64")
    g = O.poly_psf_grad(_CPU["Teff"], opd, wls, weights, 1.0, N_FOCAL, _CPU["ps_out"], G,
                        precision="c64")
    return psf.astype(np.float32), g["g_opd"].astype(np.float32)


class CpuStep:
    """The benchmark step restated on the host: the oracle's complex64 port of
    dLux's op order (the stand-in for dLux's JAX CPU path, which cannot be
    installed here), every wavelength of the step, split in contiguous blocks
    over a process pool with one single-threaded worker per host core (started
    with spawn). One call = one PSF + coefficient-gradient evaluation."""

    def __init__(self, workers=None):
        import multiprocessing as mp
        from oracle import dlux_oracle as O

        self.coeffs, self.wls, self.weights, R = make_inputs()
        T, B = O.circular_aperture(N_PUPIL, 1.0, oversample=5, secondary_diameter=0.1,
                                   spider_width=0.01, spider_angles=(0, 90, 180, 270),
                                   zernike_nolls=NOLLS)
        self.Bf = B.astype(np.float32)
        Teff = (T / np.sqrt((T ** 2).sum())).astype(np.float32)
        self.G = np.kron(R.astype(np.float32), np.ones((OVERSAMPLE, OVERSAMPLE), np.float32))
        ps_out = float(O.arcsec2rad(PSF_PIXEL_SCALE / OVERSAMPLE))
        self.workers = int(workers or os.cpu_count() or 1)
        self.blocks = [b for b in np.array_split(np.arange(N_WAVELENGTHS), self.workers)
                       if len(b)]
        saved = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS",
                                                "MKL_NUM_THREADS")}
        for k in saved:
            os.environ[k] = "1"
        try:
            self.pool = mp.get_context("spawn").Pool(
                self.workers, initializer=_cpu_worker_init,
                initargs=(T.astype(np.float32), Teff, ps_out))
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    def __call__(self):
        from oracle import dlux_oracle as O
        opd = np.tensordot(self.Bf, self.coeffs.astype(np.float32), axes=(0, 0))
        jobs = [(opd, self.wls[b], self.weights[b], self.G) for b in self.blocks]
        parts = self.pool.map(_cpu_worker, jobs)
        psf = np.sum([p[0] for p in parts], axis=0)
        g_opd = np.sum([p[1] for p in parts], axis=0)
        img = O.downsample(psf, OVERSAMPLE, mean=False)
        gc = np.tensordot(self.Bf, g_opd, axes=((1, 2), (0, 1)))
        assert np.isfinite(img).all() and np.isfinite(gc).all()
        return img, gc

    def time(self, steps, warmup):
        for _ in range(warmup):
            self()
        times = []
        for _ in range(steps):
            t0 = time.perf_counter()
            self()
            times.append(time.perf_counter() - t0)
        return times

    def close(self):
        self.pool.close()
        self.pool.join()

    def sample(self):
        return (f"all {N_WAVELENGTHS} wavelengths of the step at full 512^2 pupil / 512^2 focal "
                f"size, in {len(self.blocks)} blocks over {self.workers} single-threaded "
                "worker processes; NumPy complex64 restatement of dLux's op order (dLux/JAX "
                "is not installable here)")


def _cpu_block(job):
    """One block of the other configurations' CPU restatement (complex64 port):
    the PSF of a block of wavelengths, or with a cotangent its reverse pass."""
    from oracle import dlux_oracle as O
    T, opd, wls, weights, m, ps_out, G, offset = job
    if G is None:
        return O.poly_psf(T, opd, wls, weights, 1.0, m, ps_out, offset=offset,
                          precision="c64").astype(np.float32)
    g = O.poly_psf_grad(T, opd, wls, weights, 1.0, m, ps_out, G, offset=offset,
                        precision="c64")
    return {k: np.asarray(v, np.float32) for k, v in g.items()}


def cpu_config_baseline(name, workers=None):
    """cpu_baseline of configurations 1, 3 and 4: the oracle's complex64 port of
    dLux's op order, timed on the host cores on a bounded sample of the workload.

    cfg1: whole evaluations (1 wavelength, 256^2 -> 128^2, PSF + coefficient
          gradient) on one core; value in ms per evaluation.
    cfg3: whole evaluations: forward PSF of all 32 wavelengths, flat field, Poisson
          NLL and its cotangent, reverse pass of all 32 wavelengths (coefficient,
          amplitude with the power normalisation's chain rule, and flat-field
          gradients), wavelength blocks over a spawn pool of single-threaded
          workers; evals/s.
    cfg4: the forward and reverse pass of `workers` of the 1024 sources (all 16
          wavelengths each, one source per worker), scaled to the scene: each
          source costs the same; evals/s.
    """
    import multiprocessing as mp
    from oracle import dlux_oracle as O

    workers = int(workers or os.cpu_count() or 1)
    ps = float(O.arcsec2rad(0.02))
    saved = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS",
                                            "MKL_NUM_THREADS")}
    for k in saved:
        os.environ[k] = "1"
    try:
        pool = None if name == "cfg1" else mp.get_context("spawn").Pool(workers)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    try:
        if name == "cfg1":
            rng = np.random.default_rng(1)
            T, B = O.circular_aperture(256, 1.0, oversample=1, secondary_diameter=0.1,
                                       zernike_nolls=list(range(4, 14)))
            Teff = (T / np.sqrt((T ** 2).sum())).astype(np.float32)
            B = B.astype(np.float32)
            c = rng.normal(0, 50e-9, 10).astype(np.float32)
            R = rng.normal(size=(128, 128)).astype(np.float32)

            def one():
                opd = np.tensordot(B, c, axes=(0, 0))
                psf = _cpu_block((T, opd, [1e-6], [1.0], 128, ps, None, (0.0, 0.0)))
                g = _cpu_block((Teff, opd, [1e-6], [1.0], 128, ps, R, (0.0, 0.0)))
                return float((psf * R).sum()), np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))
            one()
            t = []
            for _ in range(20):
                t0 = time.perf_counter()
                one()
                t.append(time.perf_counter() - t0)
            return {"value": 1e3 * float(np.median(t)), "unit": "ms", "cores": 1, "kind": "port",
                    "sample": "20 whole evaluations (median) after one warm-up, one thread; "
                              "NumPy complex64 restatement of dLux's op order"}
        if name == "cfg3":
            rng = np.random.default_rng(3)
            T, B = O.circular_aperture(512, 1.0, oversample=1, secondary_diameter=0.1,
                                       zernike_nolls=list(range(4, 40)))
            A = (T * (1 + rng.normal(0, 0.01, T.shape))).astype(np.float32)
            B = B.astype(np.float32)
            c = rng.normal(0, 40e-9, 36).astype(np.float32)
            flat = (1 + rng.normal(0, 0.02, (256, 256))).astype(np.float32)
            wls = np.linspace(0.9e-6, 1.1e-6, 32)
            w = np.full(32, 1.0 / 32)
            blocks = [b for b in np.array_split(np.arange(32), workers) if len(b)]
            data = None

            def one():
                nonlocal data
                opd = np.tensordot(B, c, axes=(0, 0))
                s = 1.0 / np.sqrt((A.astype(np.float64) ** 2).sum())
                Aeff = (A * s).astype(np.float32)
                psf = np.sum(pool.map(_cpu_block, [(Aeff, opd, wls[b], w[b], 256, ps, None,
                                                    (0.0, 0.0)) for b in blocks]), axis=0)
                img = psf * flat * 1e6
                if data is None:
                    data = rng.poisson(img).astype(np.float32)
                loss = float((img - data * np.log(img)).sum())
                g_img = (1.0 - data / img).astype(np.float32)
                g_flat = g_img * psf * 1e6
                G = (g_img * flat * 1e6).astype(np.float32)
                parts = pool.map(_cpu_block, [(Aeff, opd, wls[b], w[b], 256, ps, G, (0.0, 0.0))
                                              for b in blocks])
                g_opd = np.sum([q["g_opd"] for q in parts], axis=0)
                g_eff = np.sum([q["g_amp"] for q in parts], axis=0)
                g_A = s * g_eff - s ** 3 * A * float((A * g_eff).sum())
                g_c = np.tensordot(B, g_opd, axes=((1, 2), (0, 1)))
                return loss, g_c, g_A, g_flat
            one()
            t = []
            for _ in range(3):
                t0 = time.perf_counter()
                one()
                t.append(time.perf_counter() - t0)
            return {"value": 1.0 / float(np.median(t)), "unit": "evals/s", "cores": workers,
                    "kind": "port",
                    "sample": f"3 whole evaluations (median) after one warm-up: 32 wavelengths "
                              f"in {len(blocks)} blocks over {workers} single-threaded worker "
                              "processes; NumPy complex64 restatement of dLux's op order"}
        if name == "cfg4":
            rng = np.random.default_rng(4)
            T, B = O.circular_aperture(1024, 1.0, oversample=1, secondary_diameter=0.1,
                                       zernike_nolls=list(range(4, 25)))
            Teff = (T / np.sqrt((T ** 2).sum())).astype(np.float32)
            B = B.astype(np.float32)
            c = rng.normal(0, 30e-9, 21).astype(np.float32)
            S = 1024
            pos = rng.uniform(-2, 2, (S, 2)) * np.pi / 180 / 3600
            flux = 10 ** rng.uniform(2, 6, S)
            R = rng.normal(size=(128, 128)).astype(np.float32)
            wls = np.linspace(0.8e-6, 1.2e-6, 16)
            w = np.full(16, 1.0 / 16)
            opd = np.tensordot(B, c, axes=(0, 0))
            xs = O.coord_xs(1024, 1.0 / 1024)
            X, Y = np.meshgrid(xs, xs, indexing="xy")

            def sample(srcs):
                # forward PSF and reverse pass (flux-weighted cotangent) per source
                fwd = pool.map(_cpu_block, [(T, opd, wls, w, 128, ps, None, tuple(pos[i]))
                                            for i in srcs])
                rev = pool.map(_cpu_block, [(Teff, opd, wls, w, 128, ps,
                                             (flux[i] * R).astype(np.float32), tuple(pos[i]))
                                            for i in srcs])
                img = np.sum([flux[i] * f for i, f in zip(srcs, fwd)], axis=0)
                g_flux = [float((f * R).sum()) for f in fwd]
                g_pos = [(float((q["g_opd"] * X).sum()), float((q["g_opd"] * Y).sum()))
                         for q in rev]
                return img, g_flux, g_pos
            srcs = list(range(workers))
            sample(srcs)
            t0 = time.perf_counter()
            sample(srcs)
            dt = time.perf_counter() - t0
            return {"value": 1.0 / (dt * S / len(srcs)), "unit": "evals/s", "cores": workers,
                    "kind": "port",
                    "sample": f"{len(srcs)} of the {S} sources (all 16 wavelengths each, forward "
                              f"and reverse pass, one source per single-threaded worker "
                              f"process) after one warm-up, scaled by {S}/{len(srcs)}; NumPy "
                              "complex64 restatement of dLux's op order"}
        raise ValueError(name)
    finally:
        if pool is not None:
            pool.close()
            pool.join()


def parity_sample(variant, n_lambda_sample=2):
    """Part of the CPU-baseline leg: the FP64 oracle (the checker) on the same
    wavelength sample at full size, against the public-API step on the GPU for
    those wavelengths and weights. Relative L2 errors of the 128^2 image and of
    the coefficient gradient."""
    import torch
    from oracle import dlux_oracle as O

    coeffs, wls, weights, R = make_inputs()
    T, B = O.circular_aperture(N_PUPIL, 1.0, oversample=5, secondary_diameter=0.1,
                               spider_width=0.01, spider_angles=(0, 90, 180, 270),
                               zernike_nolls=NOLLS)
    ps_out = float(O.arcsec2rad(PSF_PIXEL_SCALE / OVERSAMPLE))
    idx = np.linspace(0, N_WAVELENGTHS - 1, n_lambda_sample).astype(int)
    opd = np.tensordot(B, coeffs, axes=(0, 0))
    psf = O.poly_psf(T, opd, wls[idx], weights[idx], 1.0, N_FOCAL, ps_out)
    img_ref = O.downsample(psf, OVERSAMPLE, mean=False)
    Teff = T / np.sqrt((T ** 2).sum())
    G = np.kron(R, np.ones((OVERSAMPLE, OVERSAMPLE)))
    g = O.poly_psf_grad(Teff, opd, wls[idx], weights[idx], 1.0, N_FOCAL, ps_out, G)
    gc_ref = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))

    import dlux_gb300 as dl
    dl.set_variant(variant)
    f32 = dict(dtype=torch.float32, device="cuda")
    c = torch.as_tensor(coeffs, **f32)
    # the same aperture and basis arrays on both sides, through the public API
    optics = dl.AngularOpticalSystem(
        N_PUPIL, 1.0, [dl.TransmissiveLayer(torch.as_tensor(T, **f32), normalise=True),
                       dl.BasisLayer(torch.as_tensor(B, **f32), c)],
        N_FOCAL // OVERSAMPLE, PSF_PIXEL_SCALE, OVERSAMPLE)
    detector = dl.LayeredDetector([dl.Downsample(OVERSAMPLE)])
    _, gc, img = step(optics, detector, wls[idx], torch.as_tensor(weights[idx], **f32),
                      torch.as_tensor(R, **f32), c)
    torch.cuda.synchronize()

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))
    return {"image_rel_l2": rel(img.cpu().numpy(), img_ref),
            "grad_rel_l2": rel(gc.cpu().numpy(), gc_ref),
            "reference": "FP64 NumPy restatement of dLux's op order (the oracle)",
            "sample": f"{n_lambda_sample} of {N_WAVELENGTHS} wavelengths (first and last) at "
                      "full size through the same public API; tests/test_gpu_headline_parity.py "
                      "checks all 64"}


def run_reference(args, rank, world):
    """--impl reference: the CPU restatement of the whole step timed on the host cores."""
    if rank != 0:
        return 0
    cpu = CpuStep()
    try:
        times = cpu.time(args.steps, max(args.warmup, 0))
    finally:
        cpu.close()
    t = sum(times) / len(times)
    value = 1.0 / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (seeded PCG64)", "config": config_dict(),
        "p50_ms": statistics.median(times) * 1e3, "p99_ms": float(np.percentile(times, 99)) * 1e3,
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": cpu.workers,
                         "kind": "port", "sample": cpu.sample()},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def build_workload(variant):
    import torch
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu

    dl.set_variant(variant)
    coeffs, wls, weights, R = make_inputs()
    T, B = dlu.circular_aperture(N_PUPIL, 1.0, oversample=5, secondary_diameter=0.1,
                                 spider_width=0.01, spider_angles=(0, 90, 180, 270),
                                 zernike_nolls=NOLLS)
    c = torch.as_tensor(coeffs, dtype=torch.float32, device="cuda")
    optics = dl.AngularOpticalSystem(N_PUPIL, 1.0, [dl.TransmissiveLayer(T, normalise=True),
                                                    dl.BasisLayer(B, c)],
                                     N_FOCAL // OVERSAMPLE, PSF_PIXEL_SCALE, OVERSAMPLE)
    detector = dl.LayeredDetector([dl.Downsample(OVERSAMPLE)])
    w = torch.as_tensor(weights, dtype=torch.float32, device="cuda")
    Rt = torch.as_tensor(R, dtype=torch.float32, device="cuda")
    return optics, detector, wls, w, Rt, coeffs


def step(optics, detector, wls, w, R, c):
    """One PSF + gradient evaluation through the public API."""
    c = c.detach().requires_grad_(True)
    sys_ = optics.set("layers.BasisLayer.coefficients", c)
    psf = sys_.propagate(wls, weights=w, return_psf=True)
    img = detector.model(psf)
    loss = (img * R).sum()
    loss.backward()
    return loss.detach(), c.grad, img.detach()


def graphed_step(objs):
    """The same step captured once as a CUDA graph (dlux_gb300.graphs.GraphedStep): the
    GB300 counterpart of jax.jit of the step. Coefficients in, (loss, grad, image) out."""
    from dlux_gb300.graphs import GraphedStep
    import torch

    optics, detector, wls, w, R, coeffs = objs
    c0 = torch.as_tensor(coeffs, dtype=torch.float32, device="cuda")
    return GraphedStep(lambda c: step(optics, detector, wls, w, R, c), c0), c0


def time_gpu(args, variant, rank, world, measure_roofline=True):
    import torch
    import dlux_gb300._lib as L

    optics, detector, wls, w, R, coeffs = build_workload(variant)
    c = torch.as_tensor(coeffs, dtype=torch.float32, device="cuda")
    for _ in range(max(3, args.warmup)):
        step(optics, detector, wls, w, R, c)
    torch.cuda.synchronize()
    lib = L.load()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = lib.dlx_launch_count()
    if measure_roofline:
        L.check(lib.dlx_gemm_timing_begin())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        step(optics, detector, wls, w, R, c)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = lib.dlx_launch_count() - launches0
    gemm = None
    if measure_roofline:
        import ctypes
        tot = ctypes.c_double(0)
        cnt = ctypes.c_int(0)
        fl = ctypes.c_double(0)
        L.check(lib.dlx_gemm_timing_end(ctypes.byref(tot), ctypes.byref(cnt), ctypes.byref(fl)))
        gemm = {"total_ms": tot.value, "launches": cnt.value, "flops": fl.value}
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return {"ms_total": ms, "launches": launches, "gemm": gemm, "clocks": clk,
            "objects": (optics, detector, wls, w, R, coeffs)}


def time_graphed(args, gstep, c0, world):
    """Device throughput of the graphed step with the inputs resident (CUDA events)."""
    import torch

    for _ in range(max(3, args.warmup)):
        gstep(c0)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        gstep(c0)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms


def step_latencies(gstep, c0, n):
    """Per-step device latency of the graphed step: CUDA events around each of n
    replays (after the timed region, so its K-step number is unaffected)."""
    import torch

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(n)]
    for e0, e1 in evs:
        e0.record()
        gstep(c0)
        e1.record()
    torch.cuda.synchronize()
    return [e0.elapsed_time(e1) for e0, e1 in evs]


def time_e2e(args, gstep, world):
    """The step driven from host memory: the coefficients come from pinned host
    memory and the loss, gradient and image go back to pinned host memory every
    step. The same step is captured with its copies inside the graph
    (GraphedStep(host_io=True)), so a step is one graph launch and one wait."""
    import torch
    from dlux_gb300.graphs import GraphedStep

    host_c = gstep.static_in[0].detach().cpu().pin_memory()
    gio = GraphedStep(gstep.fn, host_c, warmup=1, host_io=True)
    for _ in range(2):
        gio(host_c)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        loss, g, img = gio(host_c)
    dt = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([dt], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dt = float(t.item())
    h2d = host_c.numel() * host_c.element_size()
    d2h = sum(o.numel() * o.element_size() for o in (loss, g, img))
    # per-step latency through the same host-driven graph (each step waits for its results)
    lat = []
    for _ in range(max(args.steps, LATENCY_SAMPLES)):
        t1 = time.perf_counter()
        gio(host_c)
        lat.append((time.perf_counter() - t1) * 1e3)
    return dt, h2d, d2h, lat


# Request streams of the serving workload: "mixed" draws every request's shape from
# the whole grid (one bucket per (N, M, L) in it); "fixed" sends one shape (512^2
# pupil, 256^2 PSF, 16 wavelengths), the case where batch shapes repeat and
# captured CUDA graphs get reused.
STREAM_SHAPES = {
    "mixed": dict(pupils=(128, 256, 512, 1024), focals=(64, 128, 256, 512),
                  min_wavelengths=1, max_wavelengths=64),
    "fixed": dict(pupils=(512,), focals=(256,), min_wavelengths=16, max_wavelengths=16),
}


def _serving_tuner(shapes="mixed"):
    """The per-(N, M) plan autotuner, tuned once over the stream's shape grid."""
    from dlux_gb300.autotune import PlanTuner

    tuner = PlanTuner()
    grid, secs = tuner.tune_grid(STREAM_SHAPES[shapes]["pupils"], STREAM_SHAPES[shapes]["focals"])
    from dlux_gb300.autotune import config_label
    return tuner, {"seconds": secs, "cache": tuner.cache_path,
                   "choices": {f"{n}x{m}": config_label(c) for (n, m), c in sorted(grid.items())},
                   "timings": {k: v for k, v in tuner.timings.items()}}


def serve_streams(args, variant, rates, n_requests, tuner=None, shapes="mixed", graphs=False):
    """One server (form `variant`, or the autotuner's per-shape choice), made
    resident for every bucket of the streams, then one seeded Poisson stream per
    arrival rate in `rates`, timed one after the other. `shapes` names the request
    mix (STREAM_SHAPES); `graphs` pads the batches of hot buckets to power-of-two
    shapes and replays them as CUDA graphs (off: every batch launches directly).
    Returns a report per rate."""
    import torch
    from dlux_gb300 import serving

    srv = serving.PSFServer(max_batch=8, n_slots=args.slots, hbm_budget=150e9, k_max=36,
                            limits=(1024, 512, 64),
                            variant=None if tuner is not None else variant,
                            tuner=tuner, timeout_s=120.0, graphs=graphs,
                            graph_after=args.graph_after)
    mix = STREAM_SHAPES[shapes]
    streams = [serving.poisson_stream(n_requests, rate, seed=SEED + 10 * i, **mix)
               for i, rate in enumerate(rates)]
    _, warm = serving.poisson_stream(max(n_requests // 4, 50), rates[0], seed=SEED + 1, **mix)
    keys = sorted({r.key for _, reqs in streams for r in reqs} | {r.key for r in warm})
    # the warm-up also launches every bucket of the timed streams once (a plan's first
    # launch is not what the stream measures)
    seen = {r.key for r in warm}
    rng = np.random.default_rng(SEED + 2)
    for n, m, L in keys:
        if (n, m, L) not in seen:
            warm.append(serving.PSFRequest(n, m, L, rng.normal(0.0, 50e-9, 4)))
    t0 = time.perf_counter()
    resident = srv.prewarm(keys)
    t_prewarm = time.perf_counter() - t0
    srv.start()
    serving.replay(srv, np.zeros(len(warm)), warm)      # warm-up: back to back
    for r in warm:
        r.result(120.0)
    out = {}
    for rate, (times, reqs) in zip(rates, streams):
        srv.completed.clear()
        srv.stats.clear()
        srv.max_queue = 0
        srv.loop_gap_max_s = 0.0
        srv.events.clear()
        srv.ex.clear_stats()
        clocks = ClockSampler(torch.cuda.current_device())
        clocks.start()
        gc.collect()
        gc.disable()        # no collector pauses inside the timed stream
        try:
            serving.replay(srv, times, reqs)
        finally:
            gc.enable()
        clk = clocks.stop()
        rep = srv.report(reqs)
        rep.update(variant=variant if tuner is None else "autotuned", rate_hz=rate,
                   requests=n_requests, buckets=len(keys), resident_buckets=resident,
                   prewarm_s=t_prewarm, stream_shapes=shapes, graphs=bool(graphs),
                   clocks=clk)
        out[rate] = rep
    srv.stop()
    srv.close()
    return out


def run_serving(args):
    """Seeded Poisson streams of mixed-shape requests through dlux_gb300.serving.

    N in {128, 256, 512, 1024}, M in {64, 128, 256, 512}, L uniform on 1..64 over
    0.8-1.2 um, 4..36 Zernike coefficients from N(0, 50 nm), 30 % of requests ask for
    the coefficient gradient of <G, PSF> with G ~ N(0, 1). Arrivals are Poisson at
    each of --rates requests/s (default: --rate), one stream per rate. Plans of every
    bucket in the streams are made resident first (within the 150 GB budget); a
    warm-up stream of a different seed runs before the timed ones. Latency is
    submit -> result on the host (pinned copies included). --stream-shapes fixed
    sends one bucket instead (N 512, M 256, L 16), and --graphs replays the
    batches of hot buckets as CUDA graphs, so the two together measure what
    captured graphs are worth.
    """
    rates = [float(r) for r in args.rates.split(",")] if args.rates else [args.rate]
    out = {}
    tuned = args.variant == "split_bf16" and not args.no_tune
    main_leg = "autotuned" if tuned else args.variant
    variants = [main_leg] + (["fp32"] if args.variant == "split_bf16" and
                             not args.no_fp32_compare else [])
    tuning = None
    for variant in variants:
        tuner = None
        if variant == "autotuned":
            tuner, tuning = _serving_tuner(args.stream_shapes)
        out[variant] = {f"{r:g}": rep for r, rep in
                        serve_streams(args, variant, rates, args.requests, tuner,
                                      args.stream_shapes, args.graphs).items()}
    main_rep = out[main_leg][f"{rates[0]:g}"]
    line = {
        "metric": "served requests/sec (mixed PSF and PSF+grad stream)",
        "value": main_rep.get("throughput_rps"), "unit": "req/s", "n_gpus": 1,
        "steps": args.requests, "warmup": max(args.requests // 4, 50),
        "ms_per_step": 1e3 / main_rep["throughput_rps"] if main_rep.get("throughput_rps")
        else None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16x3-split (fp32 accumulate)" if args.variant == "split_bf16" else "fp32",
        "data": "synthetic (seeded Poisson stream)",
        "config": {"workload": f"serving: Poisson {rates[0]:g} req/s, " + (
                       "N in 128-1024, M in 64-512, L in 1..64" if args.stream_shapes == "mixed"
                       else "N 512, M 256, L 16") + ", K in 4..36, 30% gradients",
                   "requests": args.requests, "rates_hz": rates, "max_batch": 8,
                   "stream_shapes": args.stream_shapes, "graphs": args.graphs,
                   "slots": args.slots, "graph_after": args.graph_after, "hbm_budget_gb": 150},
        "p50_ms": main_rep.get("p50_ms"), "p99_ms": main_rep.get("p99_ms"),
        "p99_ms_by_pupil": main_rep.get("p99_ms_by_pupil"),
        "clocks": main_rep["clocks"],
        "autotune": tuning,
        "serving": out,
    }
    print(json.dumps(line))
    return 0


def serving_leg(args):
    """The serving metric beside the headline line: a short stream (--serving-requests at
    --rate) through the autotuned server and the FP32 server; throughput, p50/p99,
    mean batch and CUDA-graph hit rate of each."""
    keys = ("throughput_rps", "p50_ms", "p99_ms", "p99_ms_by_pupil", "p99_queue_ms",
            "p99_service_ms", "mean_batch", "graph_hit_rate", "graph_captures",
            "capture_ms_max", "loop_gap_max_ms", "completed", "failed", "slowest", "stalls")
    tuner, _ = _serving_tuner()
    out = {"rate_hz": args.rate, "requests": args.serving_requests}
    for name, variant, t in (("split_bf16_autotuned", None, tuner), ("fp32", "fp32", None)):
        rep = serve_streams(args, variant, [args.rate], args.serving_requests, t)[args.rate]
        out[name] = {k: rep.get(k) for k in keys}
    return out


# ----------------------------------------------------------------------------
# The other measured configurations (not the default line)
# ----------------------------------------------------------------------------
def cfg_workload(name, variant):
    """(step function, metric, unit, flops per step, description) of one configuration.

    cfg1: latency of one PSF + coefficient gradient, 256^2 pupil (10% obscuration),
          Noll 4-13 ~ N(0, 50 nm), one wavelength 1 um, 128^2 PSF at 0.02", loss sum(R*PSF).
    cfg3: phase retrieval, 512^2 pupil, amplitude T(1 + N(0, 0.01)), Noll 4-39 ~ N(0, 40 nm),
          32 wavelengths 0.9-1.1 um equal weights, 256^2 detector at 0.02" with flat field
          1 + N(0, 0.02), Poisson NLL of Poisson(1e6-photon) data; gradients w.r.t.
          coefficients, amplitude and flat.
    cfg4: 1024 point sources, 1024^2 pupil (10% obscuration), Noll 4-24 ~ N(0, 30 nm),
          positions U(-2, 2)", fluxes 10^U(2, 6), 16 wavelengths 0.8-1.2 um, one 128^2 image
          at 0.02"; gradients of sum(R*image) w.r.t. positions and fluxes.
    """
    import torch
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu

    dl.set_variant(variant)
    dev = "cuda"
    f32 = dict(dtype=torch.float32, device=dev)
    if name == "cfg1":
        rng = np.random.default_rng(1)
        T, B = dlu.circular_aperture(256, 1.0, oversample=1, secondary_diameter=0.1,
                                     zernike_nolls=list(range(4, 14)))
        c0 = torch.as_tensor(rng.normal(0, 50e-9, 10), **f32)
        R = torch.as_tensor(rng.normal(size=(128, 128)), **f32)
        optics = dl.AngularOpticalSystem(256, 1.0, [dl.TransmissiveLayer(T, normalise=True),
                                                    dl.BasisLayer(B, c0)], 128, 0.02, 1)
        wls = [1e-6]

        def step(c_in):
            c = c_in.detach().requires_grad_(True)
            psf = optics.set("layers.BasisLayer.coefficients", c).propagate(wls)
            loss = (psf * R).sum()
            loss.backward()
            return loss.detach(), c.grad

        def run():
            return step(c0)
        run.step, run.c0 = step, c0
        flops = 3 * 8 * (128 * 256 ** 2 + 128 ** 2 * 256)
        return run, "PSF+grad latency", "ms", flops, "256^2 pupil, 1 lambda, 128^2 PSF"
    if name == "cfg3":
        rng = np.random.default_rng(3)
        T, B = dlu.circular_aperture(512, 1.0, oversample=1, secondary_diameter=0.1,
                                     zernike_nolls=list(range(4, 40)))
        Tn = T.cpu().numpy() if hasattr(T, "cpu") else np.asarray(T)
        A0 = torch.as_tensor(Tn * (1 + rng.normal(0, 0.01, Tn.shape)), **f32)
        c0 = torch.as_tensor(rng.normal(0, 40e-9, 36), **f32)
        flat0 = torch.as_tensor(1 + rng.normal(0, 0.02, (256, 256)), **f32)
        wls = np.linspace(0.9e-6, 1.1e-6, 32)
        optics = dl.AngularOpticalSystem(512, 1.0, [dl.TransmissiveLayer(A0, normalise=True),
                                                    dl.BasisLayer(B, c0)], 256, 0.02, 1)
        with torch.no_grad():
            psf = optics.propagate(wls) * flat0
            lam = psf * (1e6 / psf.sum())
        data = torch.poisson(lam.double(), generator=torch.Generator(device=dev).manual_seed(3)).float()
        scale = float(1e6 / psf.sum())

        def step(c_in):
            A = A0.detach().requires_grad_(True)
            c = c_in.detach().requires_grad_(True)
            flat = flat0.detach().requires_grad_(True)
            sys_ = optics.set(["layers.TransmissiveLayer.transmission",
                               "layers.BasisLayer.coefficients"], [A, c])
            det = dl.LayeredDetector([dl.ApplyPixelResponse(flat)])
            img = det.model(sys_.propagate(wls, return_psf=True)) * scale
            loss = (img - data * torch.log(img)).sum()
            loss.backward()
            return loss.detach(), c.grad, A.grad, flat.grad

        def run():
            return step(c0)
        run.step, run.c0 = step, c0
        flops = 3 * 32 * 8 * (256 * 512 ** 2 + 256 ** 2 * 512)
        return run, "phase-retrieval loss+grad evals/sec", "evals/s", flops, \
            "512^2 pupil, 36 Zernikes, 32 lambda, 256^2 detector, Poisson NLL"
    if name == "cfg4":
        rng = np.random.default_rng(4)
        T, B = dlu.circular_aperture(1024, 1.0, oversample=1, secondary_diameter=0.1,
                                     zernike_nolls=list(range(4, 25)))
        c0 = torch.as_tensor(rng.normal(0, 30e-9, 21), **f32)
        S = int(getattr(cfg_workload, "sources", 1024))
        pos0 = torch.as_tensor(rng.uniform(-2, 2, (S, 2)) * np.pi / 180 / 3600,
                               dtype=torch.float64)
        flux0 = torch.as_tensor(10 ** rng.uniform(2, 6, S), **f32)
        R = torch.as_tensor(rng.normal(size=(128, 128)), **f32)
        wls = np.linspace(0.8e-6, 1.2e-6, 16)
        optics = dl.AngularOpticalSystem(1024, 1.0, [dl.TransmissiveLayer(T, normalise=True),
                                                     dl.BasisLayer(B, c0)], 128, 0.02, 1)

        def run():
            pos = pos0.detach().requires_grad_(True)
            flux = flux0.detach().requires_grad_(True)
            img = dl.PointSources(wls, position=pos, flux=flux).model(optics)
            loss = (img * R).sum()
            loss.backward()
            return loss
        flops = 3 * S * 16 * 8 * (128 * 1024 ** 2 + 128 ** 2 * 1024)
        return run, f"scene ({S} sources) loss+grad evals/sec", "evals/s", flops, \
            f"{S} point sources, 1024^2 pupil, 16 lambda, 128^2 image"
    raise ValueError(name)


def run_fft(args):
    """Padded centred FFT propagation (layers/propagators.py FFT, utils/propagation.py:8-64):
    forward + adjoint of a batch of 16 wavelengths at N = --fft-n (1024), pad = 2, for the
    radix-2 line-FFT form and the two DFT-GEMM forms. Unit: plane transforms (forward +
    adjoint of one wavelength) per second. Roofline of the radix form: algorithmic bytes =
    input + output of every pass, (N^2 + N P) 8 + (N P + P^2) 8 per direction."""
    import torch
    from dlux_gb300 import kernels

    n, pad, L = args.fft_n, 2, 16
    P = n * pad
    rng = np.random.default_rng(5)
    x = torch.as_tensor((rng.normal(size=(L, n, n)) + 1j * rng.normal(size=(L, n, n))) / n,
                        dtype=torch.complex64, device="cuda")
    y = torch.as_tensor((rng.normal(size=(L, P, P)) + 1j * rng.normal(size=(L, P, P))) / P,
                        dtype=torch.complex64, device="cuda")
    wls = np.linspace(0.8e-6, 1.2e-6, L)
    out = {}
    for form in ("radix", "split_bf16", "fp32"):
        plan = kernels.FFTPlan(wls, n, 1.0 / n, pad, None, False, variant=form)
        for _ in range(max(3, args.warmup)):
            plan.forward(x)
            plan.adjoint(y)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            plan.forward(x)
            plan.adjoint(y)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        out[form] = {"ms_per_step": ms, "planes_per_s": L / (ms * 1e-3)}
        plan.close()
    # Comparison only (not the product path): cuFFT through torch.fft on the same
    # pruned passes -- rows N -> P (zero-padded), then columns N -> P, and the
    # adjoint's inverse transforms of the columns and rows cropped back to N.
    def cufft_step():
        t = torch.fft.fft(x, n=P, dim=-1)
        torch.fft.fft(t, n=P, dim=-2)
        u = torch.fft.ifft(y, dim=-2)[..., :n, :]
        torch.fft.ifft(u, dim=-1)[..., :n]
    for _ in range(max(3, args.warmup)):
        cufft_step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        cufft_step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    out["cufft_comparison"] = {"ms_per_step": ms, "planes_per_s": L / (ms * 1e-3),
                               "note": "torch.fft (cuFFT), same pruned row/column passes, "
                                       "no centring ramps; a library comparison, not a "
                                       "product path"}
    hbm, _, src = load_peaks()
    bytes_step = L * 2 * ((n * n + n * P) * 8 + (n * P + P * P) * 8)
    achieved = bytes_step / (out["radix"]["ms_per_step"] * 1e-3) / 1e9
    line = {"metric": "FFT propagation forward+adjoint planes/sec", "value":
            out["radix"]["planes_per_s"], "unit": "planes/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["radix"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded PCG64)",
            "config": {"workload": f"padded centred FFT, N={n}, pad={pad}, {L} wavelengths, "
                                   "forward + adjoint"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": None,
                         "peak_source": f"{src} copy bandwidth"},
            "forms": out}
    print(json.dumps(line))
    return 0


def run_ops(args):
    """The path's other operations, each forward + reverse at a representative size:
    - LCT of an ABCD system (dLux layers/abcd_propagators.py:245-370, MFTPropagator /
      FFTPropagator): 16 wavelengths, 512 -> 512, split-BF16 and FP32 GEMM forms;
    - angular-spectrum propagation (ASMPropagator, :380-459): 16 wavelengths, 512
      padded to 1024;
    - PSF convolution, mode "same" (PSF.convolve psfs.py:93-110, ApplyJitter, resolved
      sources): 16 images of 512^2 and a 33 x 33 kernel, forward and both gradients;
    - dynamic aperture (AberratedAperture on a CoordTransform): 1024^2 transmission and
      OPD of 21 Zernikes, and the coefficient gradient.
    The line's value is the time of one step of all four. Each item reports its time and
    its rate: GEMM flops for the transforms (the launches' own CUDA-event timing),
    direct-convolution flops for the convolution, pixels for the aperture."""
    import ctypes
    import torch
    from dlux_gb300 import _lib as L
    from dlux_gb300 import kernels
    from dlux_gb300.layers.abcd_propagators import lct_axes

    lib = L.load()
    rng = np.random.default_rng(11)
    Lw, n = 16, 512
    wls = np.linspace(0.8e-6, 1.2e-6, Lw)
    dev = dict(device="cuda")

    def field(b, m):
        return torch.as_tensor((rng.normal(size=(b, m, m)) + 1j * rng.normal(size=(b, m, m)))
                               / m, dtype=torch.complex64, **dev)

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        L.check(lib.dlx_gemm_timing_begin())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        tot, cnt, fl = ctypes.c_double(0), ctypes.c_int(0), ctypes.c_double(0)
        L.check(lib.dlx_gemm_timing_end(ctypes.byref(tot), ctypes.byref(cnt), ctypes.byref(fl)))
        ms = e0.elapsed_time(e1) / args.steps
        gemm = None
        if cnt.value > 0 and tot.value > 0:
            gemm = {"launches_per_step": cnt.value / args.steps,
                    "gemm_ms_per_step": tot.value / args.steps,
                    "gemm_tflops": fl.value / (tot.value * 1e-3) / 1e12}
        return ms, gemm

    hbm, bf16, src = load_peaks()
    items = {}
    # LCT: a lens of focal length 1 m followed by 1 m of free space, 1 mm -> 1 mm grids
    M = np.array([[0.0, 1.0], [-1.0, 1.0]])
    ax = lct_axes(M, wls, n, 1e-3 / n, 0.0, n, 1e-3 / n, 0.0)
    x, y = field(Lw, n), field(Lw, n)
    for form in ("split_bf16", "fp32"):
        plan = kernels.XformPlan(ax, ax, n, n, variant=form)
        ms, gemm = timed(lambda: (plan.forward(x), plan.adjoint(y)))
        items[f"lct_{form}"] = {"ms_per_step": ms, "gemm": gemm,
                                "planes_per_s": Lw / (ms * 1e-3)}
        plan.close()
    # ASM: 512 padded to 1024, 0.5 m
    xa, ya = field(Lw, n), field(Lw, 2 * n)
    plan = kernels.ASMPlan(wls, n, 2 * n, 1e-3 / n, 0.5, variant="split_bf16")
    ms, gemm = timed(lambda: (plan.forward(xa), plan.adjoint(ya)))
    items["asm_split_bf16"] = {"ms_per_step": ms, "gemm": gemm, "planes_per_s": Lw / (ms * 1e-3)}
    plan.close()
    # PSF convolution: forward and both gradients
    imgs = torch.as_tensor(rng.random((Lw, n, n)), dtype=torch.float32, **dev)
    ker = torch.as_tensor(rng.random((33, 33)), dtype=torch.float32, **dev)
    gimg = torch.as_tensor(rng.normal(size=(Lw, n, n)), dtype=torch.float32, **dev)
    ms, _ = timed(lambda: (kernels.conv2d_same(imgs, ker),
                           kernels.conv2d_same_backward(imgs, ker, gimg)))
    fl = 3 * 2.0 * Lw * n * n * 33 * 33   # forward, input gradient, kernel gradient
    ms_f, _ = timed(lambda: kernels.conv2d_same(imgs, ker))
    items["conv_33x33"] = {"ms_per_step": ms, "tflops": fl / (ms * 1e-3) / 1e12,
                           "flops_per_step": fl, "forward_ms": ms_f,
                           "forward_tflops": fl / 3 / (ms_f * 1e-3) / 1e12}
    # dynamic aperture, 1024^2, Noll 1..21
    na = 1024
    desc = kernels.aperture_desc(na, 1.0 / na, 0.5, softening=1.0)
    noll = list(range(1, 22))
    coeffs = torch.as_tensor(rng.normal(0, 30e-9, 21), dtype=torch.float32, **dev)
    g_opd = torch.as_tensor(rng.normal(size=(na, na)), dtype=torch.float32, **dev)
    ms, _ = timed(lambda: (kernels.aberrated_aperture(desc, noll, coeffs),
                           kernels.aberrated_aperture_grad(desc, noll, g_opd)))
    items["aperture_1024_21z"] = {"ms_per_step": ms, "pixels_per_s": na * na / (ms * 1e-3)}
    # the layer-by-layer path (a layer list with an explicit MFT layer does not fold into
    # one pupil): phasor, normalisation, MFT and weighted intensity kernels, their reverse
    # kernels; 512^2 pupil, Noll 4-24, 16 wavelengths, 128^2 PSF, PSF + coefficient gradient
    import dlux_gb300 as dl
    import dlux_gb300.utils as dlu
    Tl, Bl = dlu.circular_aperture(n, 1.0, oversample=1, secondary_diameter=0.1,
                                   zernike_nolls=list(range(4, 25)))
    cl = torch.as_tensor(rng.normal(0, 30e-9, 21), dtype=torch.float32, **dev)
    Rl = torch.as_tensor(rng.normal(size=(128, 128)), dtype=torch.float32, **dev)
    layered = dl.LayeredOpticalSystem(n, 1.0, [dl.TransmissiveLayer(Tl, normalise=True),
                                               dl.BasisLayer(Bl, cl),
                                               dl.MFT(128, 1e-6 / 1.0 / 4)])

    def layered_step(c_in):
        c = c_in.detach().requires_grad_(True)
        psf = layered.set("layers.BasisLayer.coefficients", c).propagate(wls)
        (psf * Rl).sum().backward()
        return (c.grad,)

    from dlux_gb300.graphs import GraphedStep
    eager_ms, _ = timed(lambda: layered_step(cl))
    graphed = GraphedStep(layered_step, cl)
    ms, gemm = timed(lambda: graphed(cl))
    items["layered_512_16l"] = {"ms_per_step": ms, "gemm": gemm, "eager_ms_per_step": eager_ms,
                                "note": "one CUDA graph per step; not in the line's value "
                                        "(path operations only)"}
    total = sum(v["ms_per_step"] for k, v in items.items()
                if k not in ("lct_fp32", "layered_512_16l"))
    lct = items["lct_split_bf16"]["gemm"] or {}
    line = {"metric": "path operations (LCT, ASM, convolution, aperture) ms per step",
            "value": total, "unit": "ms", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3-split / fp32",
            "data": "synthetic (seeded PCG64)",
            "config": {"workload": f"LCT and ASM of {Lw} wavelengths at {n}^2 (ASM padded to "
                                   f"{2 * n}), forward + adjoint; 33x33 PSF convolution of {Lw} "
                                   f"x {n}^2, forward + gradients; {na}^2 dynamic aperture, 21 "
                                   "Zernikes, + gradient"},
            "roofline": {"bound": "tensor", "kernel": "tc_cgemm (LCT)",
                         "achieved": lct.get("gemm_tflops"), "peak": bf16, "unit": "TFLOP/s",
                         "frac": (lct["gemm_tflops"] / bf16) if lct else None, "traffic": None,
                         "peak_source": f"{src} bf16 dense (burst)"},
            "items": items}
    print(json.dumps(line))
    return 0


def run_config(args):
    import torch
    import dlux_gb300._lib as L
    import ctypes

    out = {}
    variants = [args.variant] + (["fp32"] if args.variant == "split_bf16" and
                                 not args.no_fp32_compare else [])
    for variant in variants:
        run, metric, unit, flops, desc = cfg_workload(args.workload, variant)
        for _ in range(max(3, args.warmup)):
            run()
        torch.cuda.synchronize()
        lib = L.load()
        clocks = ClockSampler(torch.cuda.current_device())
        clocks.start()
        time.sleep(0.3)
        L.check(lib.dlx_gemm_timing_begin())
        times = []
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        tot, cnt, fl = ctypes.c_double(0), ctypes.c_int(0), ctypes.c_double(0)
        L.check(lib.dlx_gemm_timing_end(ctypes.byref(tot), ctypes.byref(cnt), ctypes.byref(fl)))
        clk = clocks.stop()
        t = np.array(times)
        gemm_tf = fl.value / (tot.value * 1e-3) / 1e12 if tot.value > 0 else None
        graphed, gstep = None, None
        if hasattr(run, "step"):
            # the same step replayed as one CUDA graph, device time and end to end:
            # the coefficients come from pinned host memory and every output of the
            # step (loss and gradients) goes back to pinned host memory each step
            from dlux_gb300.graphs import GraphedStep
            try:
                gstep = GraphedStep(run.step, run.c0)
            except RuntimeError as e:  # a step that cannot be captured stays eager
                gstep, graphed = None, {"capture_error": str(e)[:200]}
        if hasattr(run, "step") and gstep is not None:
            host_c = run.c0.detach().cpu().pin_memory()
            # end to end: the same step with its host copies captured in the graph
            gio = GraphedStep(run.step, host_c, warmup=1, host_io=True)
            dev_c = run.c0.detach().clone()
            gt, et = [], []
            for i in range(args.steps + 3):   # device time of the replay
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                e0.record()
                gstep(dev_c)
                e1.record()
                torch.cuda.synchronize()
                if i >= 3:
                    gt.append(e0.elapsed_time(e1))
            for i in range(args.steps + 3):   # host in -> host out
                h0 = time.perf_counter()
                outs = [o for o in gio(host_c) if o is not None]
                if i >= 3:
                    et.append((time.perf_counter() - h0) * 1e3)
            gt, et = np.array(gt), np.array(et)
            graphed = {"device_ms_p50": float(np.percentile(gt, 50)),
                       "device_ms_p99": float(np.percentile(gt, 99)),
                       "device_ms_mean": float(gt.mean()),
                       "e2e_ms_p50": float(np.percentile(et, 50)),
                       "e2e_ms_p99": float(np.percentile(et, 99)),
                       "e2e_ms_mean": float(et.mean()),
                       "h2d_bytes": host_c.numel() * host_c.element_size(),
                       "d2h_bytes": sum(o.numel() * o.element_size() for o in outs)}
        out[variant] = {"ms_mean": float(t.mean()), "ms_p50": float(np.percentile(t, 50)),
                        "ms_p99": float(np.percentile(t, 99)),
                        "evals_per_s": 1e3 / float(t.mean()),
                        "algorithmic_tflops": flops / (t.mean() * 1e-3) / 1e12,
                        "gemm_tflops": gemm_tf,
                        "gemm_share": tot.value / t.sum() if t.sum() > 0 else None,
                        "graphed": graphed, "clocks": clk}
    main = out[args.variant]
    g = main["graphed"]
    if g is not None and "device_ms_mean" in g:
        # the step as one CUDA graph (the counterpart of jax.jit of the step); the
        # eager numbers stay in "variants"
        ms, p50, p99 = g["device_ms_mean"], g["device_ms_p50"], g["device_ms_p99"]
        execution = "one CUDA graph per step (dlux_gb300.graphs.GraphedStep)"
        e2e_v = g["e2e_ms_p50"] if args.workload == "cfg1" else 1e3 / g["e2e_ms_mean"]
        e2e = {"value": e2e_v, "unit": unit, "h2d_bytes_per_step": g["h2d_bytes"],
               "d2h_bytes_per_step": g["d2h_bytes"]}
    else:
        ms, p50, p99 = main["ms_mean"], main["ms_p50"], main["ms_p99"]
        execution = "eager launches"
        e2e = None
    value = p50 if args.workload == "cfg1" else 1e3 / ms
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": args.workload != "cfg1", "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3-split (fp32 accumulate)" if args.variant == "split_bf16" else "fp32",
            "data": "synthetic (seeded PCG64)",
            "config": {"workload": f"{args.workload}: {desc}"}, "execution": execution,
            "e2e": e2e, "p50_ms": p50, "p99_ms": p99, "eager_ms_p50": main["ms_p50"],
            "clocks": main["clocks"], "variants": out,
            "cpu_baseline": None if args.no_cpu else cpu_config_baseline(args.workload)}
    print(json.dumps(line))
    return 0


def load_peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), p.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--variant", default="split_bf16", choices=["split_bf16", "fp32"])
    ap.add_argument("--no-fp32-compare", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="serving: fixed split-BF16 plans instead of the per-(N, M) autotuner")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="psf_grad",
                    choices=["psf_grad", "serving", "cfg1", "cfg3", "cfg4", "fft", "ops"])
    ap.add_argument("--requests", type=int, default=4000, help="serving: timed requests")
    ap.add_argument("--rate", type=float, default=2000.0, help="serving: arrivals per s")
    ap.add_argument("--rates", default=None,
                    help="serving: comma-separated arrival rates, one timed stream each")
    ap.add_argument("--serving-requests", type=int, default=2000,
                    help="requests of the serving leg of the default line (0: no leg)")
    ap.add_argument("--slots", type=int, default=6,
                    help="serving: concurrent stream slots (measured: 4 gives p99 2.1-4.2 ms "
                         "across runs, 6 gives 2.1-2.2 ms, 8 oversubscribes the 150 GB budget)")
    ap.add_argument("--fft-n", type=int, default=1024, help="fft: pupil side (pad 2)")
    ap.add_argument("--scene-sources", type=int, default=1024,
                    help="cfg4: point sources (1024 is the measured configuration)")
    ap.add_argument("--stream-shapes", default="mixed", choices=sorted(STREAM_SHAPES),
                    help="serving: request shapes (mixed grid, or one fixed bucket)")
    ap.add_argument("--graphs", action="store_true",
                    help="serving: pad the batches of hot buckets to power-of-two shapes and "
                         "replay them as CUDA graphs (default: every batch launches directly)")
    ap.add_argument("--graph-after", type=int, default=8,
                    help="serving: a bucket's batches are padded to power-of-two shapes and "
                         "captured as CUDA graphs after this many launches of the bucket")
    ap.add_argument("--wavelengths", type=int, default=N_WAVELENGTHS,
                    help="wavelength count (64 is the benchmark workload; smaller values "
                         "make the bounded cases used for profiling captures)")
    args = ap.parse_args()
    globals()["N_WAVELENGTHS"] = int(args.wavelengths)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    if args.workload == "serving":
        return run_serving(args) if rank == 0 else 0
    if args.workload in ("cfg1", "cfg3", "cfg4"):
        cfg_workload.sources = args.scene_sources
        return run_config(args) if rank == 0 else 0
    if args.workload == "fft":
        return run_fft(args) if rank == 0 else 0
    if args.workload == "ops":
        return run_ops(args) if rank == 0 else 0
    if world > 1:
        torch.distributed.init_process_group("nccl")

    res = time_gpu(args, args.variant, rank, world)      # eager: roofline and launch count
    eager_value = world * args.steps / (res["ms_total"] / 1e3)
    gstep, c0 = graphed_step(res["objects"])
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    ms_total = time_graphed(args, gstep, c0, world)
    clk = clocks.stop()
    ms_step = ms_total / args.steps
    value = world * args.steps / (ms_total / 1e3)
    lat_dev = step_latencies(gstep, c0, max(args.steps, LATENCY_SAMPLES))
    e2e_dt, h2d, d2h, lat_e2e = time_e2e(args, gstep, world)
    e2e_value = world * args.steps / e2e_dt

    fp32 = None
    if not args.no_fp32_compare and args.variant == "split_bf16":
        r2 = time_gpu(args, "fp32", rank, world, measure_roofline=False)
        g2, c2 = graphed_step(r2["objects"])
        ms2 = time_graphed(args, g2, c2, world)
        fp32 = {"value": world * args.steps / (ms2 / 1e3), "ms_per_step": ms2 / args.steps,
                "eager_value": world * args.steps / (r2["ms_total"] / 1e3)}

    hbm, tflops, src = load_peaks()
    g = res["gemm"]
    roofline = None
    if g and g["launches"]:
        avg_ms = g["total_ms"] / g["launches"]
        flops_launch = g["flops"] / g["launches"]
        achieved = flops_launch / (avg_ms * 1e-3) / 1e12
        roofline = {"bound": "tensor", "achieved": achieved, "peak": tflops, "unit": "TFLOP/s",
                    "frac": achieved / tflops,
                    "traffic": GEMM_DRAM_BYTES_PER_WAVELENGTH * N_WAVELENGTHS,
                    "traffic_source": "ncu DRAM bytes of the step's GEMM launches at 16 "
                                      "wavelengths (average per launch), scaled to the "
                                      "launch's wavelengths",
                    "peak_source": f"{src} bf16 dense (burst)",
                    "kernel": "tc_cgemm_kernel" if args.variant == "split_bf16" else
                              "cgemm_fp32_kernel",
                    "algorithmic_flops_per_launch": flops_launch,
                    "avg_launch_ms": avg_ms,
                    "frac_of_split_ceiling": achieved / (tflops / 3.0),
                    # GEMM time per step (eager launches, each bracketed by events) over
                    # the graphed step that `value` times
                    "gemm_share_of_step": (g["total_ms"] / args.steps) / ms_step,
                    "gemm_launches_per_step": g["launches"] / args.steps}

    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cs = CpuStep()
        try:
            times = cs.time(CPU_BASELINE_STEPS, 1)
        finally:
            cs.close()
        cpu = {"value": len(times) / sum(times), "unit": "evals/s", "cores": cs.workers,
               "kind": "port",
               "sample": f"{len(times)} whole steps after one warm-up: " + cs.sample()}
        parity = parity_sample(args.variant, 2)
    serve = None
    if rank == 0 and world == 1 and args.serving_requests > 0 and args.variant == "split_bf16":
        serve = serving_leg(args)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3-split (fp32 accumulate)" if args.variant == "split_bf16" else "fp32",
            "data": "synthetic (seeded PCG64)",
            "config": config_dict(),
            "variant": args.variant,
            "parallelism": f"replicas x{world}",
            "p50_ms": statistics.median(lat_dev),
            "p99_ms": float(np.percentile(lat_dev, 99)),
            "latency": {"device_p50_ms": statistics.median(lat_dev),
                        "device_p99_ms": float(np.percentile(lat_dev, 99)),
                        "e2e_p50_ms": statistics.median(lat_e2e),
                        "e2e_p99_ms": float(np.percentile(lat_e2e, 99)),
                        "samples": len(lat_dev),
                        "how": "graphed step replayed one at a time: CUDA events around each "
                               "replay (device), host wall time of each host-driven replay "
                               "with its pinned copies and wait (e2e)"},
            "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": res["launches"],
            "execution": "one CUDA graph per step (dlux_gb300.graphs.GraphedStep over the "
                         "public API; the same kernels as the eager step)",
            "eager_value": eager_value,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "error_vs_fp64_oracle": parity,
            "clocks": clk,
            "fp32_form": fp32,
            "speedup_vs_fp32": (value / fp32["value"]) if fp32 else None,
            "serving": serve,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
