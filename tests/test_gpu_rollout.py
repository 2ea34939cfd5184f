"""GPU parity of SingleCoreNSSolver.step / rollout against the oracle, the
reference's own goldens, and size-independent properties at full size."""
import math

import numpy as np
import pytest
import torch

from oracle import ns_oracle as O
from tests.conftest import rel_l2
from ns_solver_jax_differential_distributed_gb300.workloads import (
    PLAIN_SCALE_CENTRAL, PLAIN_SMALL, spectral_u0, theta_draw)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nsgb(cuda_lib):
    import ns_solver_jax_differential_distributed_gb300 as m
    return m


def make_solver(nsgb, N, L, nu, dt, steps, scheme, **kw):
    grid = nsgb.make_grid(N, L)
    phys = nsgb.Phys(nu=nu, mu0=0.5, sigma0=0.1, C=1.0)
    return nsgb.SingleCoreNSSolver(grid, phys, nsgb.Time(dt=dt, steps=steps), scheme, **kw)


def oracle_cfg(w, steps=None, scheme=None):
    return O.OracleConfig(N=w.N, L=w.L, nu=w.nu, dt=w.dt, steps=steps or w.steps,
                          scheme=scheme or w.scheme)


@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_config1_parity(nsgb, scheme):
    """N=128 on [0, 2pi]^2, 100 steps, dt=1e-3, seeded spectral u0 (K=8),
    3-entry theta: rel-L2 <= 1e-5 after 1 step and <= 1e-4 after 100 steps
    against the float32 oracle; the error against float64 is reported."""
    w = PLAIN_SMALL
    u0, th = w.u0(), w.theta()
    for steps, tol in ((1, 1e-5), (100, 1e-4)):
        s = make_solver(nsgb, w.N, w.L, w.nu, w.dt, steps, scheme)
        J, u = s.rollout(torch.from_numpy(u0).cuda(), torch.from_numpy(th).cuda())
        J32, u32 = O.rollout(u0, th, oracle_cfg(w, steps, scheme))
        J64, u64 = O.rollout(u0.astype(np.float64), th.astype(np.float64), oracle_cfg(w, steps, scheme))
        u = u.cpu().numpy()
        assert rel_l2(u32, u) < tol, (steps, rel_l2(u32, u))
        # u0 rows have zero y-mean, so J starts as rounding noise: absolute floor
        assert abs(float(J) - float(J32)) <= tol * abs(float(J32)) + 1e-9
        print(f"{scheme} steps={steps} relL2 vs fp32 {rel_l2(u32, u):.2e} vs fp64 {rel_l2(u64, u):.2e}"
              f" (fp32 oracle vs fp64 {rel_l2(u64, u32):.2e}); J {float(J):.6e} fp32 {float(J32):.6e} fp64 {float(J64):.6e}")


def test_step_matches_oracle_step(nsgb):
    N, L = 64, 2 * math.pi
    u0 = spectral_u0(N, 8, 5)
    th = np.array([0.9, 0.4], np.float32)
    s = make_solver(nsgb, N, L, 1e-3, 1e-3, 1, "central")
    out = s.step(torch.from_numpy(u0).cuda(), torch.from_numpy(th).cuda(), 0.25).cpu().numpy()
    cfg = O.OracleConfig(N=N, L=L, nu=1e-3, dt=1e-3, steps=1)
    ref = O.solver_step(u0, th, np.float32(0.25), cfg)
    assert rel_l2(ref, out) < 1e-6


@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_reference_scheme_study_golden(nsgb, golden, scheme):
    """Zero-IC objective / kinetic energy / max speed of the reference's
    SchemeComparisonStudy at nu=0.01 (N=128, 328 steps)."""
    row = next(r for r in golden["studies"]["scheme"] if r["scheme"] == scheme and r["nu"] == 0.01)
    s = make_solver(nsgb, 128, 1.0, row["nu"], row["dt"], row["steps"], scheme)
    J = float(s.objective(torch.tensor(row["theta"]).cuda()))
    _, u = s.rollout(torch.zeros(2, 128, 128).cuda(), torch.tensor(row["theta"]).cuda())
    u = u.double().cpu().numpy()
    assert abs(J / row["objective"] - 1) < 2e-6
    ke = 0.5 * np.sum(u[0] ** 2 + u[1] ** 2) * (1 / 128) ** 2
    assert abs(ke / row["kinetic_energy"] - 1) < 5e-6
    assert abs(np.sqrt(u[0] ** 2 + u[1] ** 2).max() / row["max_velocity"] - 1) < 2e-6


def test_reference_speed_field_golden(nsgb, golden):
    import os
    f = golden["speed_fields"][0]
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", f["file"]))
    s = make_solver(nsgb, 128, 1.0, f["nu"], f["dt"], f["steps"], "central")
    _, u = s.rollout(torch.zeros(2, 128, 128).cuda(), torch.tensor(f["theta"]).cuda())
    u = u.double().cpu().numpy()
    assert rel_l2(ref, np.sqrt(u[0] ** 2 + u[1] ** 2)) < 1e-6


def test_graph_and_direct_launch_bitwise_equal(nsgb):
    w = PLAIN_SMALL
    u0, th = (torch.from_numpy(a).cuda() for a in (w.u0(), w.theta()))
    a = make_solver(nsgb, w.N, w.L, w.nu, w.dt, 77, "central", use_graph=True).rollout(u0, th)
    b = make_solver(nsgb, w.N, w.L, w.nu, w.dt, 77, "central", use_graph=False).rollout(u0, th)
    c = make_solver(nsgb, w.N, w.L, w.nu, w.dt, 77, "central", use_graph=True).rollout(u0, th)
    assert torch.equal(a[1], b[1]) and torch.equal(a[0], b[0])
    assert torch.equal(a[1], c[1]) and torch.equal(a[0], c[0])


def test_zero_steps_and_inputs_untouched(nsgb):
    w = PLAIN_SMALL
    u0 = torch.from_numpy(w.u0()).cuda()
    keep = u0.clone()
    s = make_solver(nsgb, w.N, w.L, w.nu, w.dt, 0, "central")
    J, u = s.rollout(u0, torch.tensor([1.0, 0.5]).cuda())
    assert float(J) == 0.0 and torch.equal(u, u0)
    make_solver(nsgb, w.N, w.L, w.nu, w.dt, 3, "upwind").rollout(u0, torch.tensor([1.0, 0.5]).cuda())
    assert torch.equal(u0, keep)


def test_nan_propagates(nsgb):
    """Like the reference, non-finite input propagates (no silent repair)."""
    w = PLAIN_SMALL
    u0 = torch.from_numpy(w.u0()).cuda()
    u0[0, 3, 4] = float("nan")
    J, u = make_solver(nsgb, w.N, w.L, w.nu, w.dt, 3, "central").rollout(u0, torch.tensor([1.0, 0.5]).cuda())
    assert not torch.isfinite(u).all()


@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_full_size_N4096(nsgb, scheme):
    """N=4096: 2 steps against the oracle, then 200-step size-independent
    properties (finite, divergence bounded, determinism)."""
    w = PLAIN_SCALE_CENTRAL
    u0, th = w.u0(), w.theta()
    s2 = make_solver(nsgb, w.N, w.L, w.nu, w.dt, 2, scheme)
    J, u = s2.rollout(torch.from_numpy(u0).cuda(), torch.from_numpy(th).cuda())
    J32, u32 = O.rollout(u0, th, oracle_cfg(w, 2, scheme))
    assert rel_l2(u32, u.cpu().numpy()) < 1e-5
    assert abs(float(J) - float(J32)) <= 1e-5 * abs(float(J32)) + 1e-9
    s = make_solver(nsgb, w.N, w.L, w.nu, w.dt, w.steps, scheme)
    uu0, tth = torch.from_numpy(u0).cuda(), torch.from_numpy(th).cuda()
    Ja, ua = s.rollout(uu0, tth)
    Jb, ub = s.rollout(uu0, tth)
    assert torch.isfinite(ua).all() and torch.equal(ua, ub) and torch.equal(Ja, Jb)
    dx = w.L / w.N
    div = (torch.roll(ua[0], -1, 0) - torch.roll(ua[0], 1, 0) + torch.roll(ua[1], -1, 1)
           - torch.roll(ua[1], 1, 1)) / (2 * dx)
    assert float(div.abs().max()) < 1e-2 * float(ua.abs().max()) / dx


def test_largest_grid_N8192(nsgb):
    """N=8192 (the largest plan): 2 steps against the float32 oracle, on the
    row-streaming stencil and on the tiled one (the same bits)."""
    from ns_solver_jax_differential_distributed_gb300 import _native
    w = PLAIN_SCALE_CENTRAL
    N = 8192
    u0 = spectral_u0(N, 32, 5)
    th = theta_draw(w.nu, seed=5)
    cfg = O.OracleConfig(N=N, L=w.L, nu=float(th[2]), dt=w.dt, steps=2, scheme="central")
    J32, u32 = O.rollout(u0, th, cfg)
    plan = _native.get_plan(N, w.L, torch.device("cuda"))
    old = plan.tiles()
    outs = []
    try:
        for tiles in ((2048, 54), (64, 16)):
            plan.set_tiles(tiles[0], tiles[1], old[2], old[3])
            s = make_solver(nsgb, N, w.L, float(th[2]), w.dt, 2, "central")
            J, u = s.rollout(torch.from_numpy(u0).cuda(), torch.from_numpy(th).cuda())
            outs.append(u.cpu())
            assert rel_l2(u32, u.cpu().numpy()) < 1e-5
            assert abs(float(J) - float(J32)) <= 1e-5 * abs(float(J32)) + 1e-9
    finally:
        plan.set_tiles(*old)
    assert torch.equal(outs[0], outs[1])


def test_plan_rejects_n_beyond_max(nsgb):
    from ns_solver_jax_differential_distributed_gb300 import _native
    for N in (16384, 8, 96):
        with pytest.raises(_native.NativeError):
            _native.Plan(N, 1.0, torch.device("cuda"))


def test_runner_writes_reference_speed_field(nsgb, golden, tmp_path, monkeypatch):
    """runner.main with the reference's sample config for N=128 writes the
    reference's output file, whose content matches the speed field the
    reference shipped (runner.py:162-175); --profile times the stages."""
    import json
    import os
    from ns_solver_jax_differential_distributed_gb300 import runner
    f = golden["speed_fields"][0]
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", f["file"]))
    cfg = tmp_path / "config_N_128.json"
    cfg.write_text(json.dumps({"N": 128, "nu": 0.0001, "t": 0.5, "advection_scheme": "central"}))
    monkeypatch.chdir(tmp_path)
    out = runner.main(["--config", str(cfg), "--profile", "--profile-warmup", "1", "--profile-runs", "2"])
    assert out["path"] == "result/velocity_magnitude_single_N128.npy"
    speed = np.load(tmp_path / out["path"])
    assert speed.shape == (128, 128) and speed.dtype == np.float32
    assert rel_l2(ref, speed.astype(np.float64)) < 1e-6


def test_time_step_pipeline_matches_rollout(nsgb):
    """nsgb_time_step_pipeline (per-kernel times inside back-to-back steps,
    the roofline timing of bench.py): positive, and summing to about the
    per-step time of a graph-replayed rollout."""
    from ns_solver_jax_differential_distributed_gb300 import _native
    N, L, nu, dt, steps = 1024, 2 * math.pi, 1e-4, 2.5e-4, 64
    u0 = torch.from_numpy(spectral_u0(N, 32, 0)).cuda()
    th = torch.from_numpy(theta_draw(nu, seed=0)).cuda()
    st = _native.time_step_pipeline(u0, th, L, nu, dt, "central", steps=20)
    assert set(st) == {"stencil", "rows_fwd", "cols", "rows_inv"} and all(v > 0 for v in st.values())
    _native.op_rollout(u0, th, steps, L, nu, dt, 0, 0.5, 0.1, 1.0, True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        _native.op_rollout(u0, th, steps, L, nu, dt, 0, 0.5, 0.1, 1.0, True)
    e1.record()
    torch.cuda.synchronize()
    per_step = e0.elapsed_time(e1) / (3 * steps)
    ratio = sum(st.values()) / per_step
    assert 0.5 < ratio < 2.0, (st, per_step)
