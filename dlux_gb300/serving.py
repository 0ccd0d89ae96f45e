"""Continuous-batching PSF / PSF-gradient server on one GPU.

dLux itself has no serving loop. This module serves the same polychromatic
PSF (``OpticalSystem.propagate`` of a circular telescope with a Zernike
``BasisLayer``) to many concurrent requests.

Request. Pupil size N, PSF size M, wavelength count L on a fixed band, up
to ``k_max`` Zernike coefficients (Noll 4...), optional spectral weights, and
optionally a cotangent image for d<g_psf, PSF>/d coefficients.

Scheduling (``PSFServer``, host only, independent of the executor):
- Requests are grouped by bucket (N, M, L). Each bucket has one resident
  plan holding the cached DFT operands of its wavelengths.
- Whenever a stream slot is free, the bucket whose oldest request is the
  oldest in the queue gets the slot. Up to ``max_batch`` of its requests go
  into one batched launch. While the slots are busy, new arrivals queue up
  and form larger batches. This is continuous batching: it never waits for
  a batch to fill.
- Admission is by device memory. Resident plans, per-pupil models and slot
  workspaces are counted against ``hbm_budget``. Idle plans are evicted
  least-recently-used first. A request whose plan can never fit is rejected
  with ``ValueError``.
- Completion is polled through CUDA events with a host-side deadline.
  A batch that misses it fails its requests with ``TimeoutError``.
  Cancelled requests are dropped before launch, or their results are
  discarded after it.

Execution (``CudaExecutor``):
- Each slot has a CUDA stream, a plan workspace, a serving workspace and
  pinned staging buffers.
- A batch is one ``dlx_serve_run`` call: H2D copies, Zernike OPDs, fused
  PSF, reverse pass, coefficient gradient, D2H copies.
- With graphs on, a bucket becomes hot after ``graph_after`` launches. A batch
  of a hot bucket with R requests (n_grad of them with gradients) is padded
  to R' = the next power of two and n_grad to the next power of two (at most
  R'), with zero-weight, zero-cotangent filler objects whose results are
  dropped; after ``graph_after`` launches of the same (slot, bucket, R',
  n_grad') that call is captured as a CUDA graph and replayed from then on.
  Batches of cold buckets launch directly with their exact shapes, so a
  stream of many rarely repeated shapes pays neither for padding nor for
  captures. Each bucket has a home slot (a hash of its shape), used whenever
  it is free, so that a bucket's graphs are found again. Graphs are off by
  default: the batches are long enough (a few hundred microseconds of GPU
  work and more) that the launch overhead a graph saves is smaller than what
  padding and captures cost under load.
- A request's numbers are bit-for-bit the same alone and inside any batch.
  The kernels give each object identical arithmetic and fixed-order
  reductions.
"""

from __future__ import annotations

import collections
import ctypes
import itertools
import queue
import threading
import time

import numpy as np
import torch

from . import _lib, kernels

__all__ = ["PSFRequest", "PSFServer", "CudaExecutor", "RequestCancelled", "poisson_stream",
           "replay"]

_ids = itertools.count()
DEFAULT_BAND = (0.8e-6, 1.2e-6)


class RequestCancelled(RuntimeError):
    """The request was cancelled before its result was delivered."""


class PSFRequest:
    """One PSF (and optionally d<g_psf, PSF>/d coefficients) evaluation."""

    def __init__(self, n_pupil, n_focal, n_wavelengths, coefficients, want_grad=False,
                 g_psf=None, weights=None):
        self.id = next(_ids)
        self.n_pupil = int(n_pupil)
        self.n_focal = int(n_focal)
        self.n_wavelengths = int(n_wavelengths)
        self.coefficients = np.asarray(coefficients, np.float32).reshape(-1)
        self.want_grad = bool(want_grad)
        self.g_psf = None if g_psf is None else np.asarray(g_psf, np.float32)
        L = max(self.n_wavelengths, 1)
        self.weights = (np.full(L, 1.0 / L, np.float32) if weights is None
                        else np.asarray(weights, np.float32).reshape(-1))
        self.t_submit = None
        self.t_launch = None
        self.t_done = None
        self.psf = None
        self.grad = None
        # Result buffers, allocated (and their pages touched) here in the
        # caller's thread rather than by the scheduler when the batch retires.
        # Fresh allocations there cost the scheduler up to ~10 ms in page
        # faults and memory-map locking at times, which showed in p99.
        self._psf_out = None
        self._grad_out = None
        if 0 < self.n_focal <= 8192:
            self._psf_out = np.empty((self.n_focal, self.n_focal), np.float32)
            self._psf_out.fill(0.0)   # writes every page now
            if self.want_grad:
                self._grad_out = np.zeros(self.coefficients.size, np.float32)
        self.error = None
        self.cancelled = False
        self.done = threading.Event()

    @property
    def key(self):
        return (self.n_pupil, self.n_focal, self.n_wavelengths)

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit

    def validate(self, k_max, limits):
        n_max, m_max, l_max = limits
        if self.n_pupil <= 0 or self.n_focal <= 0 or self.n_wavelengths <= 0:
            raise ValueError("pupil, PSF and wavelength counts must be positive")
        if self.n_pupil > n_max or self.n_focal > m_max or self.n_wavelengths > l_max:
            raise ValueError(f"request {self.key} exceeds the server limits {tuple(limits)}")
        if not 0 < self.coefficients.size <= k_max:
            raise ValueError(f"between 1 and {k_max} Zernike coefficients are supported")
        if not np.all(np.isfinite(self.coefficients)):
            raise ValueError("coefficients must be finite")
        if self.weights.shape != (self.n_wavelengths,) or not np.all(np.isfinite(self.weights)):
            raise ValueError("weights must be finite with one entry per wavelength")
        if self.want_grad:
            if self.g_psf is None or self.g_psf.shape != (self.n_focal, self.n_focal):
                raise ValueError("a gradient request needs g_psf of shape (n_focal, n_focal)")
        elif self.g_psf is not None:
            raise ValueError("g_psf given without want_grad")

    def cancel(self):
        """Ask for the request to be dropped; a finished request is left as it is."""
        self.cancelled = True

    def result(self, timeout=None):
        """Block until finished; returns (psf, grad) or raises the request's error."""
        if not self.done.wait(timeout):
            raise TimeoutError(f"request {self.id} not finished within {timeout} s")
        if self.error is not None:
            raise self.error
        return self.psf, self.grad


def _finish(req, error=None):
    req.error = error
    req.t_done = time.perf_counter()
    req.done.set()


class PSFServer:
    """Continuous-batching scheduler over an executor (``CudaExecutor`` by default)."""

    def __init__(self, executor=None, max_batch=8, hbm_budget=150e9, timeout_s=30.0,
                 k_max=36, limits=(1024, 512, 64), **executor_kwargs):
        self.max_batch = int(max_batch)
        self.k_max = int(k_max)
        self.limits = tuple(int(v) for v in limits)
        if executor is None:
            executor = CudaExecutor(max_batch=self.max_batch, k_max=self.k_max,
                                    limits=self.limits, **executor_kwargs)
        self.ex = executor
        self.hbm_budget = float(hbm_budget)
        self.timeout_s = float(timeout_s)
        self.plans = collections.OrderedDict()   # key -> plan, least recently used first
        self.in_flight = collections.Counter()   # key -> batches running
        self.models = set()                      # pupil sizes with a resident model
        self.pending = collections.OrderedDict() # key -> deque of requests, oldest first
        self.inbox = queue.SimpleQueue()
        self.slots = [None] * self.ex.n_slots    # slot -> (key, requests, t_launch)
        self.running = False
        self.thread = None
        self.completed = []
        self.stats = collections.Counter()
        self.max_queue = 0
        # longest time between two scheduler iterations (the thread was busy in a
        # launch or a capture, or waiting for the interpreter lock)
        self.loop_gap_max_s = 0.0
        # host stalls of the scheduler thread over 2 ms: (start, kind, seconds, detail)
        self.events = collections.deque(maxlen=4096)
        if self.ex.fixed_bytes > self.hbm_budget:
            raise ValueError(f"slot workspaces ({self.ex.fixed_bytes / 1e9:.1f} GB) exceed the "
                             f"HBM budget ({self.hbm_budget / 1e9:.1f} GB)")

    # ---- memory accounting ----
    def resident_bytes(self):
        return (self.ex.fixed_bytes + sum(self.ex.plan_bytes(p) for p in self.plans.values()) +
                sum(self.ex.model_bytes(n) for n in self.models))

    def _need_bytes(self, key):
        extra = self.ex.plan_bytes_estimate(key)
        if key[0] not in self.models:
            extra += self.ex.model_bytes_estimate(key[0])
        return extra

    def _admit(self, key):
        """Make the bucket's plan resident; False if memory cannot be freed now."""
        if key in self.plans:
            self.plans.move_to_end(key)
            return True
        need = self._need_bytes(key)
        while self.resident_bytes() + need > self.hbm_budget:
            victim = next((k for k in self.plans if self.in_flight[k] == 0), None)
            if victim is None:
                return False
            self.ex.release_plan(victim, self.plans.pop(victim))
            self.stats["evicted"] += 1
        if key[0] not in self.models:
            self.ex.load_model(key[0])
            self.models.add(key[0])
        self.plans[key] = self.ex.create_plan(key)
        self.stats["plans_created"] += 1
        return True

    def fits(self, key):
        """Whether a plan of this bucket could ever be admitted."""
        return self.ex.fixed_bytes + self._need_bytes(key) <= self.hbm_budget

    def prewarm(self, keys):
        """Create plans (and models) for ``keys`` before serving; returns how many fit."""
        n = 0
        for key in keys:
            key = tuple(int(v) for v in key)
            if self.fits(key) and self._admit(key):
                n += 1
        return n

    # ---- public API ----
    def submit(self, req: PSFRequest) -> PSFRequest:
        req.t_submit = time.perf_counter()
        try:
            req.validate(self.k_max, self.limits)
            if not self.fits(req.key):
                raise ValueError(f"bucket {req.key} does not fit the HBM budget")
        except ValueError as e:
            self.stats["rejected"] += 1
            _finish(req, e)
            return req
        self.inbox.put(req)
        return req

    def start(self):
        if self.running:
            return self
        self.running = True
        self.thread = threading.Thread(target=self._loop, name="psf-scheduler", daemon=True)
        self.thread.start()
        return self

    def busy(self):
        return (any(s is not None for s in self.slots) or any(self.pending.values()) or
                not self.inbox.empty())

    def stop(self, drain=True):
        """Stop the scheduler; with ``drain`` wait (up to timeout_s) for queued work."""
        if drain and self.running:
            deadline = time.perf_counter() + self.timeout_s
            while self.busy() and time.perf_counter() < deadline:
                time.sleep(1e-3)
        self.running = False
        if self.thread is not None:
            self.thread.join()
            self.thread = None
        self.ex.synchronize()
        for req in self._drain_all():
            _finish(req, RuntimeError("server stopped"))

    def close(self):
        self.stop(drain=False)
        for key in list(self.plans):
            self.ex.release_plan(key, self.plans.pop(key))
        self.ex.close()

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.close()

    # ---- scheduler loop ----
    def _loop(self):
        self.ex.bind_thread()
        t_prev = time.perf_counter()
        while self.running:
            t = time.perf_counter()
            gap = t - t_prev
            t_prev = t
            if gap > self.loop_gap_max_s:
                self.loop_gap_max_s = gap
            if gap > 1e-3:
                self.stats["loop_gaps_over_1ms"] += 1
                if gap > 2e-3:
                    self.events.append((t - gap, "loop_gap", gap, None))
            progressed = self._take_inbox()
            progressed |= self._retire()
            progressed |= self._dispatch()
            if not progressed:
                if any(s is not None for s in self.slots):
                    time.sleep(20e-6)
                else:
                    try:
                        req = self.inbox.get(timeout=2e-3)
                    except queue.Empty:
                        continue
                    self._enqueue(req)

    def step(self):
        """One scheduler iteration (for callers that drive the loop themselves)."""
        return self._take_inbox() | self._retire() | self._dispatch()

    def _enqueue(self, req):
        self.pending.setdefault(req.key, collections.deque()).append(req)

    def _take_inbox(self):
        got = False
        while True:
            try:
                req = self.inbox.get_nowait()
            except queue.Empty:
                break
            self._enqueue(req)
            got = True
        if got:
            self.max_queue = max(self.max_queue, sum(len(d) for d in self.pending.values()))
        return got

    def _drain_all(self):
        out = []
        for dq in self.pending.values():
            out.extend(dq)
        self.pending.clear()
        while True:
            try:
                out.append(self.inbox.get_nowait())
            except queue.Empty:
                return out

    def _oldest_bucket(self, skip):
        # `pending` holds only buckets with queued requests, so this scan is
        # over the buckets in the queue, not over every bucket ever seen.
        best, t_best, empty = None, None, []
        for key, dq in self.pending.items():
            while dq and dq[0].cancelled:
                self.stats["cancelled"] += 1
                _finish(dq.popleft(), RequestCancelled("request cancelled"))
            if not dq:
                empty.append(key)
                continue
            if key in skip:
                continue
            if best is None or dq[0].t_submit < t_best:
                best, t_best = key, dq[0].t_submit
        for key in empty:
            del self.pending[key]
        return best

    def _dispatch(self):
        launched = False
        skip = set()
        while True:
            free = [i for i, busy in enumerate(self.slots) if busy is None]
            if not free:
                return launched
            si = free[0]
            while True:
                key = self._oldest_bucket(skip)
                if key is None:
                    return launched
                if self._admit(key):
                    break
                skip.add(key)        # memory is held by running batches: try another bucket
            home = self.ex.home_slot(key)
            if home in free:
                si = home
            dq = self.pending[key]
            reqs = []
            while dq and len(reqs) < self.max_batch:
                r = dq.popleft()
                if r.cancelled:
                    self.stats["cancelled"] += 1
                    _finish(r, RequestCancelled("request cancelled"))
                    continue
                reqs.append(r)
            if not dq:
                del self.pending[key]
            if not reqs:
                continue
            reqs.sort(key=lambda r: not r.want_grad)   # gradient requests first (stable)
            now = time.perf_counter()
            for r in reqs:
                r.t_launch = now
            try:
                self.ex.launch(si, key, self.plans[key], reqs)
                dt = time.perf_counter() - now
                if dt > 2e-3:
                    self.events.append((now, "launch", dt, [si, list(key), len(reqs)]))
            except Exception as e:  # noqa: BLE001 - delivered to the requests
                for r in reqs:
                    _finish(r, e)
                self.stats["failed"] += len(reqs)
                continue
            self.slots[si] = (key, reqs, now)
            self.in_flight[key] += 1
            self.stats["batches"] += 1
            self.stats["launched"] += len(reqs)
            launched = True

    def _retire(self):
        done_any = False
        for si, busy in enumerate(self.slots):
            if busy is None:
                continue
            key, reqs, t0 = busy
            if not self.ex.poll(si):
                if time.perf_counter() - t0 > self.timeout_s:
                    # The slot's buffers stay reserved until the device is done with them.
                    for r in reqs:
                        _finish(r, TimeoutError(f"batch on slot {si} missed its "
                                                f"{self.timeout_s} s deadline"))
                    self.stats["timed_out"] += len(reqs)
                    self.in_flight[key] -= 1
                    self.slots[si] = (None, [], float("inf"))
                    done_any = True
                continue
            if key is None:          # a timed-out batch that has finished after all
                self.slots[si] = None
                continue
            try:
                tc = time.perf_counter()
                self.ex.collect(si, reqs)
                dt = time.perf_counter() - tc
                if dt > 2e-3:
                    self.events.append((tc, "collect", dt, [si, list(key), len(reqs)]))
                err = None
            except Exception as e:  # noqa: BLE001
                err = e
            for r in reqs:
                if err is not None:
                    _finish(r, err)
                elif r.cancelled:
                    self.stats["cancelled"] += 1
                    r.psf = r.grad = None
                    _finish(r, RequestCancelled("request cancelled"))
                else:
                    _finish(r)
                    self.completed.append(r)
            self.slots[si] = None
            self.in_flight[key] -= 1
            done_any = True
        return done_any

    # ---- reporting ----
    def report(self, reqs=None):
        """Throughput and latency percentiles (JSON-serialisable)."""
        done = [r for r in (reqs if reqs is not None else self.completed)
                if r.error is None and r.t_done is not None]
        out = {"completed": len(done), "rejected": self.stats["rejected"],
               "failed": self.stats["failed"] + self.stats["timed_out"],
               "cancelled": self.stats["cancelled"], "batches": self.stats["batches"],
               "plans_created": self.stats["plans_created"], "evicted": self.stats["evicted"],
               "max_queue": self.max_queue, "resident_gb": self.resident_bytes() / 1e9,
               "loop_gap_max_ms": 1e3 * self.loop_gap_max_s,
               "loop_gaps_over_1ms": self.stats["loop_gaps_over_1ms"]}
        out.update(self.ex.stats())
        if not done:
            return out
        lat = np.array([r.latency for r in done]) * 1e3
        t0 = min(r.t_submit for r in done)
        t1 = max(r.t_done for r in done)
        wait = np.array([r.t_launch - r.t_submit for r in done]) * 1e3
        service = np.array([r.t_done - r.t_launch for r in done]) * 1e3
        out.update(throughput_rps=len(done) / max(t1 - t0, 1e-9),
                   p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
                   p99_queue_ms=float(np.percentile(wait, 99)),
                   p99_service_ms=float(np.percentile(service, 99)),
                   mean_batch=self.stats["launched"] / max(self.stats["batches"], 1))
        # the slowest requests: when they arrived (ms after the first), their shape
        # and how their latency splits into queueing and service
        worst = np.argsort(lat)[-10:][::-1]
        out["slowest"] = [{"arrival_ms": round((done[i].t_submit - t0) * 1e3, 3),
                           "latency_ms": round(float(lat[i]), 3),
                           "queue_ms": round(float(wait[i]), 3),
                           "service_ms": round(float(service[i]), 3),
                           "key": list(done[i].key), "grad": done[i].want_grad}
                          for i in worst]
        # scheduler stalls and graph captures inside the stream (ms after its start)
        evs = [e for e in list(self.events) + list(getattr(self.ex, "events", []))
               if t0 <= e[0] <= t1]
        evs.sort(key=lambda e: -e[2])
        out["stalls"] = [{"at_ms": round((e[0] - t0) * 1e3, 3), "kind": e[1],
                          "ms": round(e[2] * 1e3, 3), "detail": e[3]} for e in evs[:40]]
        by_n = collections.defaultdict(list)
        for r, l in zip(done, lat):
            by_n[r.n_pupil].append(l)
        out["p99_ms_by_pupil"] = {int(n): float(np.percentile(v, 99))
                                  for n, v in sorted(by_n.items())}
        return out


# ---------------------------------------------------------------------------
# CUDA executor
# ---------------------------------------------------------------------------

def _aligned(nbytes, device):
    """uint8 CUDA tensor of nbytes whose data pointer is 256-byte aligned (plus its owner)."""
    buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=device)
    off = (-buf.data_ptr()) % 256
    return buf, buf[off:off + nbytes]


class _Slot:
    def __init__(self, ex, index):
        dev = ex.device
        B, K = ex.max_batch, ex.k_max
        N, M, L = ex.limits
        self.index = index
        self.stream = torch.cuda.Stream(device=dev)
        self._pw, self.plan_ws = _aligned(ex.plan_ws_bytes, dev)
        self._sw, self.serve_ws = _aligned(ex.serve_ws_bytes, dev)

        def pinned(n):
            t = torch.empty(n, dtype=torch.float32).pin_memory()
            return t, t.numpy()
        self.coeffs_t, self.coeffs = pinned(B * K)
        self.weights_t, self.weights = pinned(B * L)
        self.gpsf_t, self.gpsf = pinned(B * M * M)
        self.psf_t, self.psf = pinned(B * M * M)
        self.grad_t, self.grad = pinned(B * K)
        self.event = torch.cuda.Event()
        self.current = None


class CudaExecutor:
    """Runs batches through ``dlx_serve_run`` on ``n_slots`` CUDA streams."""

    def __init__(self, max_batch=8, k_max=36, limits=(1024, 512, 64), n_slots=4,
                 diameter=1.0, psf_pixel_scale=0.02, band=DEFAULT_BAND, variant=None,
                 operand_mode=0, graphs=False, graph_after=2, max_graphs=512, device=None,
                 tuner=None, pad_batches=None):
        _lib.require_cuda()
        self.device = torch.device(device) if device is not None else \
            torch.device("cuda", torch.cuda.current_device())
        self.max_batch, self.k_max = int(max_batch), int(k_max)
        self.limits = tuple(int(v) for v in limits)
        self.diameter = float(diameter)
        self.pixel_scale = float(psf_pixel_scale) * np.pi / (180.0 * 3600.0)
        self.band = (float(band[0]), float(band[1]))
        self.variant = variant
        self.operand_mode = int(operand_mode)
        # per-(n, m) form and DFT operand from the autotuner, when no form is forced
        self.tuner = tuner if variant is None else None
        self.graphs_on = bool(graphs)
        # pad batches to power-of-two shapes (the captured graphs' shapes); on with graphs
        self.pad_batches = self.graphs_on if pad_batches is None else bool(pad_batches)
        self.graph_after = int(graph_after)
        self.max_graphs = int(max_graphs)
        N, M, L = self.limits
        with torch.cuda.device(self.device):
            self.plan_ws_bytes = self._plan_ws_bytes(N, M, L)
            b = ctypes.c_size_t(0)
            _lib.call("dlx_serve_workspace_bytes", self.max_batch, self.k_max, N, M, L,
                      ctypes.byref(b))
            self.serve_ws_bytes = int(b.value)
            self.slots = [_Slot(self, i) for i in range(int(n_slots))]
        self.n_slots = len(self.slots)
        self.fixed_bytes = self.n_slots * (self.plan_ws_bytes + self.serve_ws_bytes)
        self.models = {}
        self.graphs = collections.OrderedDict()   # (slot, key, R, G) -> CUDAGraph
        self.bucket_launches = collections.Counter()
        self.seen = collections.Counter()         # direct launches of a hot (slot, key, R, G)
        self.counts = collections.Counter()
        self.capture_s = 0.0
        self.capture_max_s = 0.0
        self.events = collections.deque(maxlen=4096)   # (start, "capture", seconds, detail)

    # ---- sizes ----
    def wavelengths(self, L):
        return np.linspace(self.band[0], self.band[1], L) if L > 1 else \
            np.array([0.5 * (self.band[0] + self.band[1])])

    def _variant(self, n, m):
        return kernels.resolve_variant(n, m, self.variant)

    def _plan_ws_bytes(self, n, m, L):
        d = _lib.PolyDesc(L, n, m, self.diameter / n, self.pixel_scale, 0.0,
                          self._variant(n, m), 0)
        b = ctypes.c_size_t(0)
        _lib.call("dlx_poly_workspace_bytes", ctypes.byref(d), self.max_batch, ctypes.byref(b))
        return int(b.value)

    def plan_bytes_estimate(self, key):
        n, m, L = key
        # two cached operand matrices per wavelength (x and y axes coincide), 8 bytes each
        return 2 * L * n * m * 8 + 4096

    def plan_bytes(self, plan):
        return plan.footprint

    def model_bytes_estimate(self, n):
        return (self.k_max + 1) * n * n * 4 + 4096

    def model_bytes(self, n):
        return self.model_bytes_estimate(n)

    # ---- resident state ----
    def bind_thread(self):
        torch.cuda.set_device(self.device)

    def load_model(self, n):
        from .utils.apertures import circular_aperture
        with torch.cuda.device(self.device):
            amp, basis = circular_aperture(n, self.diameter, oversample=3,
                                           secondary_diameter=0.1 * self.diameter,
                                           zernike_nolls=list(range(4, 4 + self.k_max)))
            amp = amp.to(self.device).contiguous()
            basis = basis.to(self.device).contiguous()
            scale = kernels.amp_norm(amp)
            torch.cuda.synchronize(self.device)
        self.models[n] = (amp, basis, scale)

    def plan_config(self, n, m):
        """(variant, operand_mode, pair) of the bucket plans of shape (n, m); pair None
        follows the process-wide paired-GEMM switch."""
        if self.tuner is not None:
            cfg = self.tuner.choose(n, m)
            return cfg["variant"], int(cfg["operand_mode"]), bool(cfg.get("pair", 0))
        return self.variant, self.operand_mode, None

    def create_plan(self, key):
        n, m, L = key
        variant, mode, pair = self.plan_config(n, m)
        with torch.cuda.device(self.device):
            return kernels.PolyPlan(self.wavelengths(L), n, self.diameter / n, m,
                                    self.pixel_scale, None, variant, self.max_batch,
                                    mode, own_workspace=False, gemm_pair=pair)

    def release_plan(self, key, plan):
        for gk in [k for k in self.graphs if k[1] == key]:
            del self.graphs[gk]
        plan.close()

    # ---- batches ----
    def home_slot(self, key):
        """The slot a bucket prefers (a fixed hash of its shape)."""
        n, m, L = key
        return (n * 7919 + m * 104729 + L * 1299709) % self.n_slots

    def padded_shape(self, R, G):
        """(R', G') of a batch of R requests, G of them with gradients."""
        if not self.pad_batches:
            return R, G

        def up(v):
            p = 1
            while p < v:
                p *= 2
            return p
        Rp = min(up(R), self.max_batch)
        Gp = 0 if G == 0 else min(up(G), Rp)
        return Rp, Gp

    def _batch_struct(self, slot, key, R, G):
        n, m, L = key
        amp, basis, scale = self.models[n]
        b = _lib.ServeBatch()
        b.n_objects, b.n_grad, b.n_coeffs = R, G, self.k_max
        b.basis, b.amp, b.amp_scale = basis.data_ptr(), amp.data_ptr(), scale.data_ptr()
        b.h_coeffs = slot.coeffs_t.data_ptr()
        b.h_weights = slot.weights_t.data_ptr()
        b.h_g_psf = slot.gpsf_t.data_ptr()
        b.h_psf = slot.psf_t.data_ptr()
        b.h_grad = slot.grad_t.data_ptr()
        b.d_work = slot.serve_ws.data_ptr()
        b.d_work_bytes = self.serve_ws_bytes
        return b

    def launch(self, si, key, plan, reqs):
        """Enqueue a batch on slot si; reqs hold the gradient requests first."""
        slot = self.slots[si]
        n, m, L = key
        G_req = sum(1 for r in reqs if r.want_grad)
        self.bucket_launches[key] += 1
        hot = self.graphs_on and self.bucket_launches[key] >= self.graph_after
        R, G = self.padded_shape(len(reqs), G_req) if hot else (len(reqs), G_req)
        K = self.k_max
        c = slot.coeffs[:R * K].reshape(R, K)
        c[:] = 0.0
        w = slot.weights[:R * L].reshape(R, L)
        w[:] = 0.0              # filler objects: zero weights, so a zero field
        for i, r in enumerate(reqs):
            c[i, :r.coefficients.size] = r.coefficients
            w[i] = r.weights
        if G:
            g = slot.gpsf[:G * m * m].reshape(G, m, m)
            for i in range(G):
                if i < G_req:
                    g[i] = reqs[i].g_psf
                else:           # a forward-only request or a filler in the gradient group
                    g[i] = 0.0
        self.counts["padded_objects"] += R - len(reqs)
        gk = (si, key, R, G)
        stream = slot.stream
        graph = self.graphs.get(gk) if hot else None
        with torch.cuda.stream(stream):
            if graph is not None:
                self.graphs.move_to_end(gk)
                graph.replay()
                self.counts["graph_replays"] += 1
            else:
                if hot:
                    self.seen[gk] += 1
                b = self._batch_struct(slot, key, R, G)
                plan.attach_workspace(slot.plan_ws)
                if hot and self.seen[gk] >= self.graph_after:
                    t0 = time.perf_counter()
                    graph = torch.cuda.CUDAGraph()
                    graph.capture_begin(capture_error_mode="thread_local")
                    try:
                        _lib.call("dlx_serve_run", plan.handle, ctypes.byref(b),
                                  stream.cuda_stream)
                    finally:
                        graph.capture_end()
                    self.graphs[gk] = graph
                    if len(self.graphs) > self.max_graphs:
                        self.graphs.popitem(last=False)
                    self.counts["graph_captures"] += 1
                    graph.replay()
                    # host time of capture, instantiation and first replay: the
                    # scheduler thread is busy for this long
                    dt = time.perf_counter() - t0
                    self.capture_s += dt
                    self.capture_max_s = max(self.capture_max_s, dt)
                    self.events.append((t0, "capture", dt, [si, list(key), R, G]))
                else:
                    _lib.call("dlx_serve_run", plan.handle, ctypes.byref(b), stream.cuda_stream)
                    self.counts["direct_launches"] += 1
            slot.event.record(stream)
        slot.current = (key, R, G_req)

    def poll(self, si):
        return self.slots[si].event.query()

    def collect(self, si, reqs):
        slot = self.slots[si]
        (n, m, L), R, G = slot.current
        psf = slot.psf[:R * m * m].reshape(R, m, m)
        grad = slot.grad[:G * self.k_max].reshape(G, self.k_max)
        for i, r in enumerate(reqs):
            if r._psf_out is not None and r._psf_out.shape == psf[i].shape:
                np.copyto(r._psf_out, psf[i])
                r.psf = r._psf_out
            else:
                r.psf = psf[i].copy()
            if i < G:
                if r._grad_out is not None:
                    np.copyto(r._grad_out, grad[i, :r.coefficients.size])
                    r.grad = r._grad_out
                else:
                    r.grad = grad[i, :r.coefficients.size].copy()
        slot.current = None

    def synchronize(self):
        torch.cuda.synchronize(self.device)

    def stats(self):
        total = self.counts["graph_replays"] + self.counts["direct_launches"] + \
            self.counts["graph_captures"]
        caps = self.counts["graph_captures"]
        return {"graph_hit_rate": self.counts["graph_replays"] / max(total, 1),
                "graphs": len(self.graphs), "graph_captures": caps,
                "capture_ms_mean": 1e3 * self.capture_s / caps if caps else None,
                "capture_ms_max": 1e3 * self.capture_max_s if caps else None,
                "padded_objects": self.counts["padded_objects"]}

    def clear_stats(self):
        self.counts.clear()
        self.events.clear()
        self.capture_s = self.capture_max_s = 0.0

    def close(self):
        self.synchronize()
        self.graphs.clear()
        self.models.clear()


# ---------------------------------------------------------------------------
# Synthetic workload
# ---------------------------------------------------------------------------

def poisson_stream(n_requests, rate_hz, seed, pupils=(128, 256, 512, 1024),
                   focals=(64, 128, 256, 512), max_wavelengths=64, k_range=(4, 36),
                   grad_fraction=0.3, coeff_sigma=50e-9, min_wavelengths=1):
    """Seeded request stream: arrival offsets (s) of a Poisson process and the requests.

    Shapes are drawn uniformly from ``pupils`` x ``focals`` x
    min_wavelengths..max_wavelengths, the coefficient count uniformly from
    ``k_range``, coefficients from N(0, coeff_sigma) m; a fraction ``grad_fraction``
    asks for gradients with an N(0, 1) cotangent image. One pupil, one focal side
    and min_wavelengths == max_wavelengths give a stream of a single bucket.
    """
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, n_requests)
    times = np.concatenate([[0.0], np.cumsum(gaps[1:])])
    reqs = []
    for _ in range(n_requests):
        n = int(rng.choice(pupils))
        m = int(rng.choice(focals))
        L = int(rng.integers(min_wavelengths, max_wavelengths + 1))
        k = int(rng.integers(k_range[0], k_range[1] + 1))
        grad = bool(rng.random() < grad_fraction)
        g = rng.standard_normal((m, m), dtype=np.float32) if grad else None
        reqs.append(PSFRequest(n, m, L, rng.normal(0.0, coeff_sigma, k), grad, g))
    return times, reqs


def replay(server, times, reqs, wait_s=None):
    """Submit ``reqs`` at their arrival offsets and wait for all of them."""
    t0 = time.perf_counter()
    for t, r in zip(times, reqs):
        delay = t0 + t - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        server.submit(r)
    limit = server.timeout_s if wait_s is None else wait_s
    for r in reqs:
        r.done.wait(limit)
    return reqs
