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
        alone = serve.Request(r.rid, 0.0, r.N, r.steps, r.kind, r.seed, nu=r.nu, dt=r.dt, theta=r.theta)
        srv1 = serve.Server(hbm_budget=2e9, slice_steps=5, grad_workers=1)
        (a,), _ = srv1.run([alone], realtime=False)
        assert a.J == r.J, (r.rid, a.J, r.J)
        if r.kind == "grad":
            assert np.array_equal(a.grad, r.grad)
        else:
            assert torch.equal(a.u_final, r.u_final)


def test_admission_respects_budget(serve):
    reqs = _trace(serve, 16)
    srv = serve.Server(hbm_budget=6e7, slice_steps=16, grad_workers=1)
    peak = []
    orig = srv.run

    done, trace = orig(reqs, realtime=False)
    assert len(done) == len(reqs)
    assert srv.used == pytest.approx(0.0)


def test_summary(serve):
    reqs = _trace(serve, 12)
    srv = serve.Server(hbm_budget=2e9, slice_steps=16, grad_workers=1)
    done, _ = srv.run(reqs, realtime=False)
    s = serve.summarize(reqs, done, 1.0)
    assert s["completed"] == len(reqs) and s["p99_latency_s"] >= s["p50_latency_s"] >= 0
