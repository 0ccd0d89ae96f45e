"""Autotuner for the launch configuration of poly plans, per (n_in, n_out).

The serving loop groups requests into buckets of (pupil size, focal size,
wavelength count). Each bucket runs on one poly plan, and a plan fixes how
its GEMMs run:
- ``variant``: the split-BF16 tensor-core form (128 x 128 complex tiles fed
  by TMA) or the FP32 CUDA-core form (128 x 64 shared-memory tiles, one
  CTA per tile and batch element), which can win for tiny transforms that
  leave most SMs idle;
- ``operand_mode``: the DFT operand streamed from cached matrices by TMA
  (0), or generated inside the GEMM's CTAs (1), which halves the operand
  bytes and the plan's memory;
- ``pair``: for the streamed operand, 256 x 128 tiles on clusters of two
  CTAs (cta_group::2 MMAs, each CTA loading half of the A tile) instead of
  128 x 128 tiles on one CTA -- a candidate only where a GEMM of the plan
  has an even number of 128-column tiles;
- ``split_k`` (plans with their own workspace only): whether GEMMs whose
  tiles leave most SMs idle split K, at the count fixed at plan creation.

The tile shapes searched are therefore 128 x 128 on one CTA and 256 x 128 on
a CTA pair. Narrower tiles are not candidates: on GB300 a tcgen05 MMA with
N = 64 (or 32) columns takes 50.8 cycles where the full rate would be 32, so
a 128 x 64 tile spends 1.59x the MMA time per flop; wider tiles do not fit
the main and cross accumulators in tensor memory.

``PlanTuner.choose(n, m)`` times each candidate on a probe batch (the
one-sweep PSF + gradient of ``probe_objects`` objects at ``probe_wavelengths``
wavelengths) with CUDA events, keeps the fastest, and caches the choice in
memory and in a JSON file keyed by the device name. The file is given by
``cache_path``, else ``$DLUX_GB300_TUNE_CACHE``, else
``~/.cache/dlux_gb300/tune.json``. All candidates agree with the FP64 oracle
within 1e-5, so the choice affects speed and memory only.
"""

from __future__ import annotations

import json
import os
import threading
import time

import numpy as np

__all__ = ["PlanTuner", "candidate_configs", "config_label"]


def _tiles(side):
    return (int(side) + 127) // 128


def candidate_configs(n, m, tensor_cores=True, own_workspace=False):
    """Configurations worth timing for an (n_in, n_out) plan."""
    fp32 = {"variant": "fp32", "operand_mode": 0, "pair": 0, "split_k": 1}
    if not tensor_cores:
        return [fp32]
    out = [{"variant": "split_bf16", "operand_mode": 0, "pair": 0, "split_k": 1}]
    if _tiles(n) % 2 == 0 or _tiles(m) % 2 == 0:
        out.append({"variant": "split_bf16", "operand_mode": 0, "pair": 1, "split_k": 1})
    out.append({"variant": "split_bf16", "operand_mode": 1, "pair": 0, "split_k": 1})
    if own_workspace:
        out.append({"variant": "split_bf16", "operand_mode": 0, "pair": 0, "split_k": 0})
    return out + [fp32]


def config_label(cfg):
    label = f"{cfg['variant']}/op{cfg['operand_mode']}"
    if cfg.get("pair"):
        label += "/pair"
    if not cfg.get("split_k", 1):
        label += "/nosplit"
    return label


def _default_cache_path():
    env = os.environ.get("DLUX_GB300_TUNE_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "dlux_gb300", "tune.json")


class PlanTuner:
    """Chooses a poly plan's arithmetic form and DFT operand per (n_in, n_out)."""

    def __init__(self, cache_path=None, probe_wavelengths=8, probe_objects=4, iters=5,
                 diameter=1.0, psf_pixel_scale_rad=1e-7, timer=None, device_name=None,
                 own_workspace=False):
        self.cache_path = cache_path if cache_path is not None else _default_cache_path()
        self.probe_wavelengths = int(probe_wavelengths)
        self.probe_objects = int(probe_objects)
        self.iters = int(iters)
        self.diameter = float(diameter)
        self.pixel_scale = float(psf_pixel_scale_rad)
        self._timer = timer            # (n, m, config) -> seconds; None: time on the GPU
        # plans with their own workspace may split K; shared-workspace (serving) plans do not
        self.own_workspace = bool(own_workspace)
        self._device = device_name
        self._lock = threading.Lock()
        self._mem = {}
        self.timings = {}              # key -> {config label: seconds}, for reports

    # ---- cache ----
    def device_name(self):
        if self._device is None:
            import torch
            self._device = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
        return self._device

    def _key(self, n, m):
        ws = "own" if self.own_workspace else "shared"
        return f"{self.device_name()}|{ws}|{int(n)}|{int(m)}"

    def _load_file(self):
        try:
            with open(self.cache_path) as f:
                data = json.load(f)
            return data if isinstance(data, dict) else {}
        except (OSError, ValueError):
            return {}

    def _store_file(self, key, cfg):
        data = self._load_file()
        data[key] = cfg
        d = os.path.dirname(self.cache_path)
        try:
            if d:
                os.makedirs(d, exist_ok=True)
            tmp = f"{self.cache_path}.{os.getpid()}.tmp"
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, self.cache_path)
        except OSError:
            pass  # an unwritable cache only costs a re-tune

    # ---- choice ----
    def choose(self, n, m):
        """{"variant", "operand_mode", "pair", "split_k"} for a poly plan of this shape."""
        key = self._key(n, m)
        with self._lock:
            if key in self._mem:
                return dict(self._mem[key])
            cached = self._load_file().get(key)
            if isinstance(cached, dict) and all(k in cached for k in
                                                ("variant", "operand_mode", "pair", "split_k")):
                self._mem[key] = cached
                return dict(cached)
            cfg = self._tune(n, m)
            self._mem[key] = cfg
            self._store_file(key, cfg)
            return dict(cfg)

    def _tune(self, n, m):
        if self._timer is None:
            from . import kernels
            tc = kernels.tensor_core_available()
        else:
            tc = True
        results, configs = {}, {}
        for cfg in candidate_configs(n, m, tc, self.own_workspace):
            label = config_label(cfg)
            try:
                t = self._timer(n, m, cfg) if self._timer else self._time_gpu(n, m, cfg)
            except Exception:  # a candidate that cannot run here is skipped
                continue
            results[label] = float(t)
            configs[label] = cfg
        if not results:
            raise RuntimeError(f"no plan configuration runs for n={n}, m={m}")
        self.timings[self._key(n, m)] = results
        best = min(results, key=results.get)
        return dict(configs[best], seconds=results[best])

    def _time_gpu(self, n, m, cfg):
        import torch
        from . import kernels

        from . import _lib

        L, R = self.probe_wavelengths, self.probe_objects
        wls = np.linspace(0.8e-6, 1.2e-6, L)
        # shared-workspace (serving) plans do not split K: probe those likewise
        lib = _lib.load()
        if not self.own_workspace:
            _lib.check(lib.dlx_set_split_k(0))
        try:
            plan = kernels.PolyPlan(wls, n, self.diameter / n, m, self.pixel_scale,
                                    variant=cfg["variant"], max_objects=R,
                                    operand_mode=cfg["operand_mode"],
                                    gemm_pair=bool(cfg.get("pair", 0)),
                                    split_k=bool(cfg.get("split_k", 1)))
        finally:
            if not self.own_workspace:
                _lib.check(lib.dlx_set_split_k(1))
        try:
            rng = np.random.default_rng(n * 7919 + m)
            dev = dict(dtype=torch.float32, device="cuda")
            yy, xx = np.mgrid[:n, :n]
            r2 = ((xx - (n - 1) / 2) ** 2 + (yy - (n - 1) / 2) ** 2) / (n / 2) ** 2
            amp = torch.as_tensor((r2 <= 1.0).astype(np.float32), **dev)
            scale = kernels.amp_norm(amp)
            objs = []
            for _ in range(R):
                objs.append(dict(
                    amp=amp, amp_scale=scale,
                    opd=torch.as_tensor(rng.normal(0, 30e-9, (n, n)), **dev),
                    weights=torch.full((L,), 1.0 / L, **dev),
                    psf=torch.empty((m, m), **dev),
                    g_psf=torch.as_tensor(rng.normal(size=(m, m)), **dev),
                    g_opd=torch.empty((n, n), **dev)))
            for _ in range(2):
                plan.forward_backward_objects(objs)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(self.iters):
                plan.forward_backward_objects(objs)
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) * 1e-3 / self.iters
        finally:
            plan.close()

    def tune_grid(self, pupils, focals):
        """Choose for every (n, m) of a grid up front (a server's start-up)."""
        t0 = time.perf_counter()
        out = {(int(n), int(m)): self.choose(n, m) for n in pupils for m in focals}
        return out, time.perf_counter() - t0
