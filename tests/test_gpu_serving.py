"""Serving loop on the GPU: parity with the oracle, and each request's result is bit for bit
the same alone and inside mixed batches (direct launches and CUDA-graph replays).

Tolerances against the FP64 oracle: PSF and coefficient gradient relative L2 <= 1e-5.
"""

import ctypes
import time

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu

K = 10
LIMITS = (128, 64, 4)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_server(**kw):
    from dlux_gb300.serving import PSFServer
    kw.setdefault("max_batch", 4)
    kw.setdefault("n_slots", 2)
    return PSFServer(hbm_budget=20e9, k_max=K, limits=LIMITS, timeout_s=60.0, **kw)


def drive(server, reqs, limit_s=60.0):
    """Run the scheduler on this thread until every request has finished."""
    deadline = time.perf_counter() + limit_s
    while not all(r.done.is_set() for r in reqs):
        server.step()
        assert time.perf_counter() < deadline, "serving batches did not finish"
    for r in reqs:
        if r.error is not None:
            raise r.error


def requests(seed, n_req=12):
    from dlux_gb300.serving import PSFRequest
    rng = np.random.default_rng(seed)
    shapes = [(128, 64, 3), (64, 32, 2), (128, 32, 4)]
    out = []
    for i in range(n_req):
        n, m, L = shapes[i % len(shapes)]
        k = int(rng.integers(3, K + 1))
        grad = bool(i % 3 == 0)
        g = rng.standard_normal((m, m)).astype(np.float32) if grad else None
        w = rng.dirichlet(np.ones(L)).astype(np.float32)
        out.append(PSFRequest(n, m, L, rng.normal(0, 50e-9, k), grad, g, w))
    return out


def clone(reqs):
    from dlux_gb300.serving import PSFRequest
    return [PSFRequest(r.n_pupil, r.n_focal, r.n_wavelengths, r.coefficients, r.want_grad,
                       r.g_psf, r.weights) for r in reqs]


def test_serving_matches_oracle(cuda):
    from dlux_gb300.serving import PSFRequest
    s = make_server(graphs=False)
    rng = np.random.default_rng(11)
    n, m, L = 128, 64, 3
    c = rng.normal(0, 50e-9, K)
    G = rng.standard_normal((m, m)).astype(np.float32)
    w = rng.dirichlet(np.ones(L)).astype(np.float32)
    r = s.submit(PSFRequest(n, m, L, c, True, G, w))
    drive(s, [r])
    psf, grad = r.result(0)
    amp, basis, _ = (t.cpu().numpy() for t in s.ex.models[n])
    coeffs = np.asarray(c, np.float32).astype(np.float64)
    opd = O.eval_basis(basis.astype(np.float64), coeffs)
    wls = s.ex.wavelengths(L)
    ps = s.ex.pixel_scale
    ref = O.poly_psf(amp, opd, wls, w, 1.0, m, ps)
    amp_eff = amp.astype(np.float64) / np.sqrt((amp.astype(np.float64) ** 2).sum())
    g_opd = O.poly_psf_grad(amp_eff, opd, wls, w, 1.0, m, ps, G)["g_opd"]
    gref = basis.reshape(K, -1).astype(np.float64) @ g_opd.reshape(-1)
    e_psf, e_grad = rel(psf, ref), rel(grad, gref)
    print(f"serving vs oracle: psf {e_psf:.2e}, grad {e_grad:.2e}")
    assert e_psf < 1e-5 and e_grad < 1e-5
    s.close()


@pytest.mark.parametrize("variant", ["fp32", "split_bf16"])
def test_alone_vs_mix_bitwise(cuda, variant):
    base = requests(5)
    alone_srv = make_server(max_batch=1, n_slots=1, graphs=False, variant=variant)
    alone = clone(base)
    for r in alone:
        alone_srv.submit(r)
        drive(alone_srv, [r])
    alone_srv.close()

    mix_srv = make_server(max_batch=4, n_slots=2, graphs=True, graph_after=1, variant=variant)
    rounds = []
    for _ in range(2):     # first round captures graphs, second replays them
        mix = clone(base)
        for r in mix:
            mix_srv.submit(r)
        drive(mix_srv, mix)
        rounds.append(mix)
    rep = mix_srv.report()
    mix_srv.close()
    assert rep["batches"] < 2 * len(base), "requests were not batched"
    assert rep["graph_captures"] > 0 and rep["graph_hit_rate"] > 0
    for mix in rounds:
        for a, b in zip(alone, mix):
            assert np.array_equal(a.psf, b.psf), f"psf of request {a.key} differs in a batch"
            if a.want_grad:
                assert np.array_equal(a.grad, b.grad), f"grad of {a.key} differs in a batch"


def test_threaded_stream(cuda):
    from dlux_gb300.serving import poisson_stream, replay
    s = make_server(max_batch=4, n_slots=3).start()
    times, reqs = poisson_stream(120, 2000.0, seed=2, pupils=(64, 128), focals=(32, 64),
                                 max_wavelengths=4, k_range=(3, K))
    replay(s, times, reqs)
    s.stop()
    rep = s.report()
    s.close()
    print("threaded stream:", rep)
    assert rep["completed"] == len(reqs)
    assert all(np.isfinite(r.psf).all() for r in reqs)
    assert all(r.grad is not None for r in reqs if r.want_grad)


def test_serve_run_rejects_bad_batches(cuda):
    from dlux_gb300 import _lib
    s = make_server(graphs=False)
    key = (64, 32, 2)
    s.prewarm([key])
    plan = s.plans[key]
    slot = s.ex.slots[0]
    plan.attach_workspace(slot.plan_ws)

    def run(**over):
        b = s.ex._batch_struct(slot, key, 1, 0)
        for k, v in over.items():
            setattr(b, k, v)
        _lib.call("dlx_serve_run", plan.handle, ctypes.byref(b),
                  torch.cuda.current_stream().cuda_stream)

    with pytest.raises(ValueError, match="n_objects"):
        run(n_objects=0)
    with pytest.raises(ValueError, match="n_objects"):
        run(n_objects=5)
    with pytest.raises(ValueError, match="n_grad"):
        run(n_grad=2)
    with pytest.raises(ValueError, match="aligned"):
        run(d_work=slot.serve_ws.data_ptr() + 4)
    with pytest.raises(ValueError, match="needed"):
        run(d_work_bytes=1024)
    with pytest.raises(ValueError, match="h_g_psf"):
        run(n_grad=1, h_g_psf=None)
    run()                                  # the unmodified batch is accepted
    torch.cuda.synchronize()
    s.close()


def test_autotuned_server_alone_vs_mix_and_oracle(cuda, tmp_path):
    """A server whose bucket plans take their form and DFT operand from the
    autotuner: the tuner times every candidate and records a choice, results
    stay bit-identical alone and in a mix, and match the oracle."""
    from dlux_gb300.autotune import PlanTuner
    tuner = PlanTuner(cache_path=str(tmp_path / "tune.json"), probe_wavelengths=2,
                      probe_objects=2, iters=2)
    base = requests(6)
    shapes = {(r.n_pupil, r.n_focal) for r in base}
    grid, secs = tuner.tune_grid(sorted({n for n, _ in shapes}), sorted({m for _, m in shapes}))
    print("autotuned:", {k: (v["variant"], v["operand_mode"]) for k, v in grid.items()},
          f"in {secs:.2f} s;", tuner.timings)
    for cfg in grid.values():
        assert cfg["variant"] in ("split_bf16", "fp32") and cfg["operand_mode"] in (0, 1)
    assert all(len(t) >= 1 for t in tuner.timings.values())

    alone_srv = make_server(max_batch=1, n_slots=1, graphs=False, tuner=tuner)
    alone = clone(base)
    for r in alone:
        alone_srv.submit(r)
        drive(alone_srv, [r])
    alone_srv.close()
    mix_srv = make_server(max_batch=4, n_slots=2, graphs=True, graph_after=1, tuner=tuner)
    mix = clone(base)
    for r in mix:
        mix_srv.submit(r)
    drive(mix_srv, mix)
    mix_srv.close()
    for a, b in zip(alone, mix):
        assert np.array_equal(a.psf, b.psf)
        if a.want_grad:
            assert np.array_equal(a.grad, b.grad)
    # one request against the oracle
    r = next(x for x in alone if x.want_grad)
    s = make_server(graphs=False, tuner=tuner)
    s.prewarm([(r.n_pupil, r.n_focal, r.n_wavelengths)])
    amp, basis, _ = (t.cpu().numpy() for t in s.ex.models[r.n_pupil])
    c = np.zeros(K)
    c[:r.coefficients.size] = np.asarray(r.coefficients, np.float32)
    opd = O.eval_basis(basis.astype(np.float64), c)
    wls = s.ex.wavelengths(r.n_wavelengths)
    ref = O.poly_psf(amp, opd, wls, r.weights, 1.0, r.n_focal, s.ex.pixel_scale)
    s.close()
    assert rel(r.psf, ref) < 1e-5
