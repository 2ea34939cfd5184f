"""Serving with continuous batching: every request completes, and each result
is the same alone and in the mix (bit for bit)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import serve
    return serve


def _trace(serve, n=40):
    return serve.make_trace(rate=400.0, duration=n / 400.0, seed=11, sizes=(32, 64, 128),
                            steps_range=(8, 60), p_grad=0.3)


def test_mix_completes_and_equals_alone(serve):
    reqs = _trace(serve)
    assert len(reqs) >= 20 and any(r.kind == "grad" for r in reqs)
    srv = serve.Server(hbm_budget=2e9, slice_steps=7, max_active_cells=3 * 128 * 128, grad_workers=2)
    done, trace = srv.run(reqs, realtime=False)
    assert len(done) == len(reqs)
    assert all(np.isfinite(r.J) for r in done)
    assert srv.used == pytest.approx(0.0)
    assert max(t[2] for t in trace) > 1, "requests were never batched together"
    picks = [r for r in reqs if r.kind == "forward"][:3] + [r for r in reqs if r.kind == "grad"][:2]
    for r in picks:
        alone = serve.Request(r.rid, 0.0, r.N, r.steps, r.kind, r.seed, nu=r.nu, dt=r.dt, scheme=r.scheme,
                              theta=r.theta)
        srv1 = serve.Server(hbm_budget=2e9, slice_steps=5, grad_workers=1)
        (a,), _ = srv1.run([alone], realtime=False)
        assert a.J == r.J, (r.rid, a.J, r.J)
        if r.kind == "grad":
            assert np.array_equal(a.grad, r.grad)
        else:
            assert torch.equal(a.u_final, r.u_final)


def test_admission_respects_budget(serve):
    """A budget that holds only a few requests: every request still
    completes, requests had to wait for memory, and the bytes in flight never
    exceeded the budget."""
    reqs = _trace(serve, 16)
    srv = serve.Server(hbm_budget=1.0, slice_steps=16, grad_workers=1)
    need = [srv._grad_bytes(r) if r.kind == "grad" else srv._fwd_bytes(r) for r in reqs]
    srv.budget = budget = 1.5 * max(need)  # room for the largest request and a little more
    assert budget < sum(need)
    done, trace = srv.run(reqs, realtime=False)
    assert len(done) == len(reqs) and all(r.status == "ok" for r in done)
    assert 0 < srv.peak_used <= budget
    assert max(t[1] for t in trace) > 0, "the budget never held a request back"
    assert srv.used == pytest.approx(0.0)


def test_failures_are_isolated(serve):
    """One request with a NaN in its initial state (status "nonfinite"), one
    whose device allocation fails (status "failed") and one cancelled before it
    runs: every other request completes with the bits of an undisturbed run."""
    clean = _trace(serve, 30)
    srv0 = serve.Server(hbm_budget=2e9, slice_steps=7, max_active_cells=3 * 128 * 128, grad_workers=2)
    ref, _ = srv0.run(clean, realtime=False)
    ref = {r.rid: r for r in ref}

    reqs = _trace(serve, 30)
    fwd = [r for r in reqs if r.kind == "forward"]
    grd = [r for r in reqs if r.kind == "grad"]
    nan_f, nan_g, boom, boom_g, gone = fwd[1], grd[0], fwd[3], grd[1], fwd[5]
    srv = serve.Server(hbm_budget=2e9, slice_steps=7, max_active_cells=3 * 128 * 128, grad_workers=2)
    for r in (nan_f, nan_g):
        u0 = srv.u0.get(r.N, r.seed).clone()
        u0[0, 2, 3] = float("nan")
        r.u0 = u0
    real_alloc = srv._alloc

    def alloc(r, shape, dtype):
        if r.rid in (boom.rid, boom_g.rid):
            raise torch.cuda.OutOfMemoryError("injected allocation failure")
        return real_alloc(r, shape, dtype)

    srv._alloc = alloc
    srv.cancel(gone.rid)
    done, _ = srv.run(reqs, realtime=False)
    assert len(done) == len(reqs)
    by = {r.rid: r for r in done}
    assert by[nan_f.rid].status == "nonfinite" and by[nan_g.rid].status == "nonfinite"
    for x in (boom, boom_g):
        assert by[x.rid].status == "failed" and "injected" in by[x.rid].error
    assert by[gone.rid].status == "cancelled"
    assert srv.used == pytest.approx(0.0)
    for rid, r in by.items():
        if rid in (nan_f.rid, nan_g.rid, boom.rid, boom_g.rid, gone.rid):
            continue
        assert r.status == "ok" and r.J == ref[rid].J, rid
        if r.kind == "grad":
            assert np.array_equal(r.grad, ref[rid].grad), rid
        else:
            assert torch.equal(r.u_final, ref[rid].u_final), rid
    s = serve.summarize(reqs, done, 1.0)
    assert s["statuses"] == {"ok": len(reqs) - 5, "nonfinite": 2, "failed": 2, "cancelled": 1}


def _clean_run(serve, n):
    srv = serve.Server(hbm_budget=2e9, slice_steps=7, max_active_cells=3 * 128 * 128, grad_workers=2)
    ref, _ = srv.run(_trace(serve, n), realtime=False)
    return {r.rid: r for r in ref}


def _assert_like(r, ref):
    assert r.status == "ok" and r.J == ref.J, r.rid
    if r.kind == "grad":
        assert np.array_equal(r.grad, ref.grad), r.rid
    else:
        assert torch.equal(r.u_final, ref.u_final), r.rid


def test_bad_requests_fail_alone(serve):
    """Requests with arguments the solver refuses (an unsupported N, an
    unknown scheme, dt = 0, a u0 of the wrong shape, theta of 4 entries) fail
    on arrival with their reason; a float64 theta is taken as float32; every
    other request completes with the bits of an undisturbed run."""
    ref = _clean_run(serve, 30)
    reqs = _trace(serve, 30)
    fwd = [r for r in reqs if r.kind == "forward"]
    grd = [r for r in reqs if r.kind == "grad"]
    bad = {fwd[0].rid: "N=100 unsupported", grd[0].rid: "scheme", fwd[2].rid: "dt must be",
           fwd[4].rid: "u0 must be", grd[1].rid: "theta must have"}
    fwd[0].N = 100
    grd[0].scheme = "lax-wendroff"
    fwd[2].dt = 0.0
    fwd[4].u0 = torch.zeros(2, fwd[4].N // 2, fwd[4].N // 2, device="cuda")
    grd[1].theta = np.array([1.0, 0.5, 1e-3, 7.0], np.float32)
    f64 = fwd[6]
    f64.theta = np.asarray(f64.theta, np.float64)
    srv = serve.Server(hbm_budget=2e9, slice_steps=7, max_active_cells=3 * 128 * 128, grad_workers=2)
    done, _ = srv.run(reqs, realtime=False)
    assert len(done) == len(reqs)
    assert srv.used == pytest.approx(0.0)
    for r in done:
        if r.rid in bad:
            assert r.status == "failed" and bad[r.rid].lower() in r.error.lower(), (r.rid, r.error)
        else:
            _assert_like(r, ref[r.rid])


def test_failed_tick_fails_only_its_requests(serve, monkeypatch):
    """A batched tick whose call reports an error (injected on the first
    forward tick and the first gradient tick) fails the requests in that tick
    only; the server serves on, and every later request completes with the
    bits of an undisturbed run."""
    from ns_solver_jax_differential_distributed_gb300 import _native
    ref = _clean_run(serve, 30)
    real_check = _native.check
    hit = set()

    def check(name, status):
        real_check(name, status)
        if name in ("nsgb_ensemble_advance", "nsgb_grad_batch_advance") and name not in hit:
            hit.add(name)
            raise RuntimeError(f"injected failure of {name}")

    monkeypatch.setattr(_native, "check", check)
    srv = serve.Server(hbm_budget=2e9, slice_steps=7, max_active_cells=3 * 128 * 128,
                       max_active_grad_cells=2 * 128 * 128)
    reqs = _trace(serve, 30)
    done, _ = srv.run(reqs, realtime=False)
    torch.cuda.synchronize()
    assert hit == {"nsgb_ensemble_advance", "nsgb_grad_batch_advance"}
    assert len(done) == len(reqs)
    assert srv.used == pytest.approx(0.0)
    failed = [r for r in done if r.status == "failed"]
    assert failed and all("injected" in r.error for r in failed)
    assert {r.kind for r in failed} == {"forward", "grad"}
    assert {r.kind for r in done if r.status == "ok"} == {"forward", "grad"}
    for r in done:
        if r.status != "failed":
            _assert_like(r, ref[r.rid])


@pytest.mark.parametrize("grad_mode", ["batched", "workers"])
def test_stop_suspends_and_resume_gives_the_same_bits(serve, monkeypatch, grad_mode):
    """Server.stop() in the middle of a run suspends the active requests to
    host memory and returns the rest as queued; a new server given them
    finishes every request with the bits of an uninterrupted run.  A
    checkpoint whose launch shapes no longer match is refused."""
    from ns_solver_jax_differential_distributed_gb300 import _native
    ref = _clean_run(serve, 30)
    kw = dict(hbm_budget=2e9, slice_steps=7, max_active_cells=3 * 128 * 128,
              max_active_grad_cells=2 * 128 * 128, grad_slice_ops=16, grad_mode=grad_mode, grad_workers=2)
    srv = serve.Server(**kw)
    real_check = _native.check
    trigger = "nsgb_grad_batch_advance" if grad_mode == "batched" else "nsgb_ensemble_advance"
    calls = [0]

    def check(name, status):
        real_check(name, status)
        if name == trigger:
            calls[0] += 1
            if calls[0] == 3:
                srv.stop()

    monkeypatch.setattr(_native, "check", check)
    reqs = _trace(serve, 30)
    done, _ = srv.run(reqs, realtime=False)
    monkeypatch.setattr(_native, "check", real_check)
    assert calls[0] == 3 and len(done) == len(reqs)
    assert srv.used == pytest.approx(0.0)
    sus = [r for r in done if r.status == "suspended"]
    rest = [r for r in done if r.status in ("suspended", "queued")]
    kinds = {"forward", "grad"} if grad_mode == "batched" else {"forward"}
    assert {r.kind for r in sus} == kinds
    assert all(0 < r.resume["progress"] for r in sus)
    assert any(r.status == "queued" for r in rest)
    # a checkpoint written under other launch shapes is refused
    odd = sus[0]
    saved = odd.resume
    odd.resume = dict(saved, shapes=((0, 0, 0, 0),) + tuple(saved["shapes"][1:]))
    srv2 = serve.Server(**kw)
    done2, _ = srv2.run(rest, realtime=False)
    assert srv2.used == pytest.approx(0.0)
    by = {r.rid: r for r in done2}
    assert by[odd.rid].status == "failed" and "launch shapes" in by[odd.rid].error
    odd.resume = saved
    (again,), _ = serve.Server(**kw).run([odd], realtime=False)
    final = {r.rid: r for r in done if r.status not in ("suspended", "queued")}
    final.update(by)
    final[odd.rid] = again
    assert len(final) == len(reqs)
    for rid, r in final.items():
        _assert_like(r, ref[rid])
        assert r.resume is None


def test_batched_and_worker_gradients_agree(serve):
    """Gradient requests served by the batched path (several in flight at
    once, work split into uneven slices) and by worker threads running
    nsgb_rollout_grad give the same bits."""
    kw = dict(hbm_budget=2e9, slice_steps=7, max_active_cells=3 * 128 * 128)
    a = serve.Server(grad_mode="batched", grad_slice_ops=5, **kw)
    da, trace = a.run(_trace(serve, 30), realtime=False)
    b = serve.Server(grad_mode="workers", grad_workers=2, **kw)
    db, _ = b.run(_trace(serve, 30), realtime=False)
    assert max(t[3] for t in trace) > 1, "gradient requests were never batched together"
    ga = {r.rid: r for r in da if r.kind == "grad"}
    gb = {r.rid: r for r in db if r.kind == "grad"}
    assert len(ga) >= 5 and ga.keys() == gb.keys()
    for rid in ga:
        assert ga[rid].status == gb[rid].status == "ok"
        assert ga[rid].J == gb[rid].J and np.array_equal(ga[rid].grad, gb[rid].grad), rid
    with pytest.raises(ValueError):
        serve.Server(grad_mode="threads")


def test_summary(serve):
    reqs = _trace(serve, 12)
    srv = serve.Server(hbm_budget=2e9, slice_steps=16, grad_workers=1)
    done, _ = srv.run(reqs, realtime=False)
    s = serve.summarize(reqs, done, 1.0)
    assert s["completed"] == len(reqs) and s["p99_latency_s"] >= s["p50_latency_s"] >= 0
