"""Host logic of the serving loop, on CPU with a fake executor.

The fake executor answers PSF = sum(coefficients) * ones and grad = 2 * coefficients,
completes a batch when the test releases it, and reports plan sizes so that admission
and eviction can be checked without a GPU. Every failure here is made on the host.
"""

import collections
import threading
import time

import numpy as np
import pytest

from dlux_gb300.serving import PSFRequest, PSFServer, RequestCancelled, poisson_stream


class FakePlan:
    def __init__(self, key, nbytes):
        self.key, self.bytes, self.closed = key, nbytes, False


class FakeExecutor:
    def __init__(self, n_slots=2, fixed_bytes=1000, auto_complete=True, fail_on=None):
        self.n_slots = n_slots
        self.fixed_bytes = fixed_bytes
        self.auto_complete = auto_complete
        self.fail_on = fail_on or set()
        self.batches = []                 # (slot, key, [request ids])
        self.running = {}                 # slot -> (key, reqs)
        self.released = set()
        self.models = []
        self.closed_plans = []

    # sizes: a plan of (n, m, L) takes n*m*L bytes, a model n bytes
    def plan_bytes_estimate(self, key):
        n, m, L = key
        return n * m * L

    def plan_bytes(self, plan):
        return plan.bytes

    def model_bytes_estimate(self, n):
        return n

    def model_bytes(self, n):
        return n

    def bind_thread(self):
        pass

    def load_model(self, n):
        self.models.append(n)

    def create_plan(self, key):
        return FakePlan(key, self.plan_bytes_estimate(key))

    def release_plan(self, key, plan):
        plan.closed = True
        self.closed_plans.append(key)

    def home_slot(self, key):
        return sum(key) % self.n_slots

    def launch(self, si, key, plan, reqs):
        assert not plan.closed
        if key in self.fail_on:
            raise RuntimeError(f"injected launch failure for {key}")
        self.batches.append((si, key, [r.id for r in reqs]))
        self.running[si] = (key, reqs)
        if self.auto_complete:
            self.released.add(si)

    def poll(self, si):
        return si in self.released

    def release(self, si=None):
        for s in (list(self.running) if si is None else [si]):
            self.released.add(s)

    def collect(self, si, reqs):
        key, batch = self.running.pop(si)
        self.released.discard(si)
        m = key[1]
        for r in reqs:
            r.psf = np.full((m, m), r.coefficients.sum(), np.float32)
            if r.want_grad:
                r.grad = 2 * r.coefficients

    def synchronize(self):
        pass

    def stats(self):
        return {}

    def close(self):
        pass


def req(n=8, m=4, L=2, k=3, grad=False, seed=0):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((m, m)).astype(np.float32) if grad else None
    return PSFRequest(n, m, L, rng.standard_normal(k), grad, g)


def server(ex=None, **kw):
    kw.setdefault("hbm_budget", 1e9)
    kw.setdefault("k_max", 8)
    kw.setdefault("limits", (64, 32, 8))
    kw.setdefault("max_batch", 4)
    return PSFServer(executor=ex or FakeExecutor(), **kw)


def run_until_idle(s, limit=1000):
    for _ in range(limit):
        s.step()
        if not s.busy():
            return
    raise AssertionError("scheduler did not go idle")


def test_results_and_batching_fifo():
    ex = FakeExecutor(n_slots=1, auto_complete=False)
    s = server(ex, max_batch=3)
    a = [s.submit(req(seed=i)) for i in range(7)]
    s.step()                                  # slot 0 takes the first 3
    assert [b[2] for b in ex.batches] == [[a[0].id, a[1].id, a[2].id]]
    s.step()                                  # slot busy: nothing new
    assert len(ex.batches) == 1
    ex.release()
    s.step()                                  # retire, then the next 3 in order
    assert ex.batches[-1][2] == [a[3].id, a[4].id, a[5].id]
    ex.release()
    s.step()
    ex.release()
    s.step()
    for r in a:
        psf, grad = r.result(0)
        assert psf.shape == (4, 4) and np.allclose(psf, r.coefficients.sum())
        assert grad is None
    assert s.report()["completed"] == 7


def test_oldest_bucket_first_and_grad_first():
    ex = FakeExecutor(n_slots=1, auto_complete=False)
    s = server(ex)
    x = s.submit(req(n=8))
    y = s.submit(req(n=16))
    z = s.submit(req(n=8, grad=True))
    s.step()
    # bucket of x (oldest) goes first and takes z with it; the gradient request leads
    assert ex.batches[0][1] == (8, 4, 2)
    assert ex.batches[0][2] == [z.id, x.id]
    ex.release()
    s.step()
    assert ex.batches[1][2] == [y.id]
    ex.release()
    s.step()
    assert np.allclose(z.result(0)[1], 2 * z.coefficients)


@pytest.mark.parametrize("bad, match", [
    (dict(n=-1), "positive"),
    (dict(L=0), "positive"),
    (dict(n=128), "exceeds"),
    (dict(k=9), "coefficients"),
    (dict(k=0), "coefficients"),
])
def test_malformed_requests_rejected(bad, match):
    s = server()
    r = s.submit(req(**bad))
    with pytest.raises(ValueError, match=match):
        r.result(0)
    assert s.report()["rejected"] == 1
    assert not s.busy()


def test_malformed_payloads_rejected():
    s = server()
    r = PSFRequest(8, 4, 2, [np.nan, 1.0])
    with pytest.raises(ValueError, match="finite"):
        s.submit(r).result(0)
    r = PSFRequest(8, 4, 2, [1.0], want_grad=True, g_psf=np.zeros((3, 3)))
    with pytest.raises(ValueError, match="g_psf"):
        s.submit(r).result(0)
    r = PSFRequest(8, 4, 2, [1.0], weights=[1.0, 2.0, 3.0])
    with pytest.raises(ValueError, match="weights"):
        s.submit(r).result(0)
    r = PSFRequest(8, 4, 2, [1.0], g_psf=np.zeros((4, 4)))
    with pytest.raises(ValueError, match="without"):
        s.submit(r).result(0)


def test_admission_evicts_least_recently_used_idle_plan():
    ex = FakeExecutor(n_slots=1, fixed_bytes=100)
    # plans: (8,4,2)=64 B, (16,4,2)=128 B, (8,8,1)=64 B, models 8/16 B
    s = server(ex, hbm_budget=100 + 64 + 128 + 24)
    for key in [(8, 4, 2), (16, 4, 2)]:
        s.submit(req(n=key[0], m=key[1], L=key[2]))
        run_until_idle(s)
    assert list(s.plans) == [(8, 4, 2), (16, 4, 2)]
    s.submit(req(n=8, m=8, L=1))
    run_until_idle(s)
    assert ex.closed_plans == [(8, 4, 2)]
    assert list(s.plans) == [(16, 4, 2), (8, 8, 1)]
    assert s.resident_bytes() <= s.hbm_budget
    assert s.report()["evicted"] == 1


def test_admission_waits_for_running_batches():
    ex = FakeExecutor(n_slots=2, fixed_bytes=100, auto_complete=False)
    s = server(ex, hbm_budget=100 + 128 + 16 + 128 + 8 - 1)
    a = s.submit(req(n=16, m=4, L=2))     # 128 B plan
    s.step()
    b = s.submit(req(n=8, m=8, L=2))      # 128 B: does not fit while a's plan is busy
    s.step()
    assert len(ex.batches) == 1 and not b.done.is_set()
    ex.release(0)
    s.step()                              # a retires, its plan is evicted, b launches
    assert a.result(0)[0] is not None
    assert ex.batches[-1][1] == (8, 8, 2)
    ex.release()
    s.step()
    assert b.result(0)[0] is not None


def test_never_fitting_bucket_rejected():
    ex = FakeExecutor(fixed_bytes=100)
    s = server(ex, hbm_budget=200)
    r = s.submit(req(n=64, m=32, L=8))
    with pytest.raises(ValueError, match="HBM budget"):
        r.result(0)


def test_workspaces_over_budget_rejected():
    with pytest.raises(ValueError, match="exceed"):
        server(FakeExecutor(fixed_bytes=10), hbm_budget=5)


def test_timeout_fails_batch_and_frees_slot_later():
    ex = FakeExecutor(n_slots=1, auto_complete=False)
    s = server(ex, timeout_s=0.02)
    r = s.submit(req())
    s.step()
    time.sleep(0.03)
    s.step()
    with pytest.raises(TimeoutError):
        r.result(0)
    nxt = s.submit(req(seed=5))
    s.step()
    assert not nxt.done.is_set() and len(ex.batches) == 1   # slot still reserved
    ex.release()
    s.step()                                 # the late batch finishes: slot freed
    s.step()
    ex.release()
    s.step()
    assert nxt.result(0)[0] is not None
    assert s.report()["failed"] == 1


def test_cancel_pending_and_in_flight():
    ex = FakeExecutor(n_slots=1, auto_complete=False)
    s = server(ex, max_batch=1)
    a = s.submit(req(seed=1))
    b = s.submit(req(seed=2))
    c = s.submit(req(seed=3))
    s.step()                 # a in flight
    a.cancel()
    b.cancel()
    ex.release()
    s.step()
    with pytest.raises(RequestCancelled):
        a.result(0)
    with pytest.raises(RequestCancelled):
        b.result(0)
    assert [x[2] for x in ex.batches] == [[a.id], [c.id]]   # b never launched
    ex.release()
    s.step()
    assert c.result(0)[0] is not None
    assert s.report()["cancelled"] == 2


def test_launch_failure_is_delivered_and_server_continues():
    ex = FakeExecutor(fail_on={(8, 4, 2)})
    s = server(ex)
    bad = s.submit(req(n=8))
    good = s.submit(req(n=16))
    run_until_idle(s)
    with pytest.raises(RuntimeError, match="injected"):
        bad.result(0)
    assert good.result(0)[0] is not None


def test_threaded_stream_with_failing_producer():
    """A producer thread that raises mid-stream: its earlier requests still complete."""
    ex = FakeExecutor(n_slots=3)
    s = server(ex, max_batch=4, limits=(64, 32, 8)).start()
    times, reqs = poisson_stream(200, 20000.0, seed=3, pupils=(8, 16), focals=(4, 8),
                                 max_wavelengths=4, k_range=(1, 8))
    submitted = []
    errors = []

    def producer():
        try:
            for i, r in enumerate(reqs):
                if i == 150:
                    raise RuntimeError("producer crashed")
                submitted.append(s.submit(r))
        except RuntimeError as e:
            errors.append(e)

    t = threading.Thread(target=producer)
    t.start()
    t.join()
    for r in submitted:
        r.result(5.0)
    s.stop()
    assert errors and len(submitted) == 150
    rep = s.report()
    assert rep["completed"] == 150 and rep["p99_ms"] >= rep["p50_ms"] > 0
    # every request answered with its own numbers
    for r in submitted:
        assert np.allclose(r.psf, r.coefficients.sum())
        if r.want_grad:
            assert np.allclose(r.grad, 2 * r.coefficients)
    # no batch mixes buckets, none exceeds max_batch
    by_id = {r.id: r for r in submitted}
    for _, key, ids in ex.batches:
        assert 1 <= len(ids) <= 4
        assert all(by_id[i].key == key for i in ids)


def test_stop_fails_queued_requests():
    ex = FakeExecutor(n_slots=1, auto_complete=False)
    s = server(ex)
    a = s.submit(req(seed=1))
    s.step()
    b = s.submit(req(n=16))
    ex.release()
    s.stop(drain=False)
    with pytest.raises(RuntimeError, match="stopped"):
        b.result(0)
    assert not a.done.is_set() or a.error is None


def test_poisson_stream_is_seeded():
    t1, r1 = poisson_stream(50, 2000.0, seed=7)
    t2, r2 = poisson_stream(50, 2000.0, seed=7)
    assert np.array_equal(t1, t2)
    assert [r.key for r in r1] == [r.key for r in r2]
    assert all(np.array_equal(a.coefficients, b.coefficients) for a, b in zip(r1, r2))
    assert abs(len(r1) / t1[-1] - 2000.0) < 1000.0
    ks = collections.Counter(r.n_pupil for r in r1)
    assert set(ks) <= {128, 256, 512, 1024}


def test_fixed_shape_stream_has_one_bucket():
    _, reqs = poisson_stream(40, 2000.0, seed=5, pupils=(512,), focals=(256,),
                             min_wavelengths=16, max_wavelengths=16)
    assert {r.key for r in reqs} == {(512, 256, 16)}
    assert any(r.want_grad for r in reqs) and not all(r.want_grad for r in reqs)


def test_bucket_goes_to_its_home_slot_when_free():
    ex = FakeExecutor(n_slots=3, auto_complete=False)
    srv = PSFServer(executor=ex, max_batch=4, hbm_budget=1e9)
    a, b = req(n=8, m=4, L=2), req(n=8, m=4, L=3)      # homes (14 % 3, 15 % 3) = (2, 0)
    srv.submit(a)
    srv.submit(b)
    srv.step()
    slots = {tuple(ids): si for si, key, ids in ex.batches}
    assert slots[(a.id,)] == 2 and slots[(b.id,)] == 0
    # with its home slot busy, a bucket takes another free slot
    c = req(n=8, m=4, L=2, seed=1)
    srv.submit(c)
    srv.step()
    assert ex.batches[-1][0] == 1 and ex.batches[-1][2] == [c.id]
    ex.release()
    srv.step()
    srv.close()


def test_padded_batch_shapes():
    from dlux_gb300.serving import CudaExecutor
    ex = CudaExecutor.__new__(CudaExecutor)
    ex.pad_batches, ex.max_batch = True, 8
    assert [ex.padded_shape(r, 0) for r in range(1, 9)] == \
        [(1, 0), (2, 0), (4, 0), (4, 0), (8, 0), (8, 0), (8, 0), (8, 0)]
    assert ex.padded_shape(3, 1) == (4, 1) and ex.padded_shape(3, 3) == (4, 4)
    assert ex.padded_shape(5, 3) == (8, 4) and ex.padded_shape(8, 8) == (8, 8)
    ex.pad_batches = False
    assert ex.padded_shape(5, 3) == (5, 3)
