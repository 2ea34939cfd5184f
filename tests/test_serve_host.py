"""Host logic of the serving loop and the optimiser study (no GPU): the
request trace, the summary statistics and the optimiser specification."""
import numpy as np
import pytest

from ns_solver_jax_differential_distributed_gb300 import optimization, serve


def test_trace_is_seeded_and_shaped():
    a = serve.make_trace(rate=200.0, duration=5.0, seed=7)
    b = serve.make_trace(rate=200.0, duration=5.0, seed=7)
    assert [(r.arrival, r.N, r.steps, r.kind) for r in a] == [(r.arrival, r.N, r.steps, r.kind) for r in b]
    assert 800 < len(a) < 1200  # Poisson, 200/s for 5 s
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0) and arr[-1] < 5.0
    assert {r.N for r in a} <= {128, 256, 512, 1024, 2048}
    assert all(100 <= r.steps <= 2000 for r in a)
    frac_grad = np.mean([r.kind == "grad" for r in a])
    assert 0.2 < frac_grad < 0.4
    for r in a[:20]:
        assert r.theta.shape == (3,) and r.cells == r.N * r.N * r.steps and r.latency is None


def test_summarize_counts_and_percentiles():
    reqs = serve.make_trace(rate=100.0, duration=1.0, seed=3, sizes=(64,), steps_range=(10, 10), p_grad=0.0)
    for i, r in enumerate(reqs):
        r.t_done = r.arrival + 0.01 * (i + 1)
    s = serve.summarize(reqs, reqs, wall=2.0)
    assert s["offered"] == s["completed"] == len(reqs)
    assert s["solves_per_s"] == pytest.approx(len(reqs) / 2.0)
    lat = [0.01 * (i + 1) for i in range(len(reqs))]
    assert s["p50_latency_s"] == pytest.approx(np.percentile(lat, 50))
    assert s["p99_latency_s"] == pytest.approx(np.percentile(lat, 99))
    assert s["forward_equiv_cell_steps_per_s"] == pytest.approx(64 * 64 * 10 * len(reqs) / 2.0)


def test_optimizer_specs():
    cfgs = optimization.default_configs()
    assert [c["name"] for c in cfgs] == ["Adam (lr=0.01)", "Adam (lr=0.001)", "SGD (lr=0.1)", "RMSprop (lr=0.01)"]
    from ns_solver_jax_differential_distributed_gb300 import _native
    a = optimization.adam(0.01).native()
    assert a.kind == _native.OPT_ADAM and a.learning_rate == pytest.approx(0.01) and a.b1 == pytest.approx(0.9)
    assert optimization.sgd(0.1).native().kind == _native.OPT_SGD
    r = optimization.rmsprop(0.01).native()
    assert r.kind == _native.OPT_RMSPROP and r.decay == pytest.approx(0.9) and r.eps == pytest.approx(1e-8)
    with pytest.raises(ValueError):
        optimization.OptimizerSpec("lamb", 0.1).native()


def test_trace_time_step_is_the_reference_stable_step():
    """Each request's dt is SimConfig.dt's rule (NS_solver.py:75-79) for its N
    and nu, rounded through float32, with upwind advection by default."""
    reqs = serve.make_trace(rate=100.0, duration=1.0, seed=5)
    for r in reqs:
        dx = 2 * np.pi / r.N
        expect = float(np.float32(min(0.4 * dx / 4.0, dx * dx / (4 * r.nu))))
        assert r.dt == expect == serve.stable_dt(r.N, 2 * np.pi, r.nu)
        assert r.scheme == "upwind"
    fixed = serve.make_trace(rate=100.0, duration=0.2, seed=5, dt=1e-3, scheme="central")
    assert all(r.dt == 1e-3 and r.scheme == "central" for r in fixed)


def test_summarize_counts_only_ok_results():
    reqs = serve.make_trace(rate=100.0, duration=0.5, seed=4, sizes=(64,), steps_range=(10, 10), p_grad=0.0)
    for i, r in enumerate(reqs):
        r.t_done = r.arrival + 0.1
        r.status = ["ok", "nonfinite", "failed", "cancelled"][i % 4]
    s = serve.summarize(reqs, reqs, wall=1.0)
    n_ok = sum(r.status == "ok" for r in reqs)
    assert s["completed"] == n_ok and s["solves_per_s"] == pytest.approx(n_ok)
    assert sum(s["statuses"].values()) == len(reqs) and s["statuses"]["ok"] == n_ok


def test_summarize_reports_unfinished_requests_apart():
    """Requests a run hands back unfinished ("suspended" with a checkpoint,
    "queued" without) appear in the status counts, never as completed."""
    reqs = serve.make_trace(rate=100.0, duration=0.5, seed=6, sizes=(64,), steps_range=(10, 10), p_grad=0.0)
    for i, r in enumerate(reqs):
        r.status = ["ok", "suspended", "queued"][i % 3]
        r.t_done = r.arrival + 0.2 if r.status == "ok" else None
    s = serve.summarize(reqs, reqs, wall=1.0)
    n_ok = sum(r.status == "ok" for r in reqs)
    assert s["completed"] == n_ok
    assert s["statuses"] == {k: sum(r.status == k for r in reqs) for k in ("ok", "suspended", "queued")}
    assert s["p50_latency_s"] == pytest.approx(0.2)
