"""Pin the CPU oracle against the reference's own shipped outputs.

The reference cannot run here (JAX is absent); its ``result/`` artefacts are
its outputs, extracted into ``tests/golden`` by ``make_golden.py``.  These
tests show the oracle reproduces them, so the GPU parity tests that compare
against the oracle compare against the reference's algorithm.
"""
import math

import numpy as np
import pytest

from oracle import ns_oracle as O
from tests.conftest import rel_l2


def _cfg(row, N=None):
    return O.OracleConfig(N=N or row["N"], L=row["L"], nu=row["nu"], dt=row["dt"],
                          steps=row["steps"], scheme=row["scheme"])


def _ke(u, dx):
    return 0.5 * np.sum(u[0].astype(np.float64) ** 2 + u[1].astype(np.float64) ** 2) * dx * dx


@pytest.mark.parametrize("idx", range(6))
def test_scheme_study_objective_energy_speed(golden, idx):
    """studies.py SchemeComparisonStudy: J, kinetic energy and max |u| for
    central/upwind at nu in {0.005, 0.01, 0.05} (N=128, zero IC)."""
    row = golden["studies"]["scheme"][idx]
    if row["steps"] > 800:
        pytest.skip("long case covered by the viscosity study test")
    cfg = _cfg(row)
    J, u = O.rollout(np.zeros((2, 128, 128), np.float32), np.array(row["theta"], np.float32), cfg)
    assert abs(float(J) / row["objective"] - 1) < 1e-6
    assert abs(_ke(u, cfg.dx) / row["kinetic_energy"] - 1) < 5e-6
    speed = np.sqrt(u[0].astype(np.float64) ** 2 + u[1] ** 2)
    assert abs(speed.max() / row["max_velocity"] - 1) < 1e-6


@pytest.mark.parametrize("nu", [0.001, 0.005])
def test_viscosity_study_objective(golden, nu):
    row = next(r for r in golden["studies"]["viscosity"] if r["nu"] == nu)
    cfg = _cfg(row)
    J, u = O.rollout(np.zeros((2, 128, 128), np.float32), np.array(row["theta"], np.float32), cfg)
    assert abs(float(J) / row["objective"] - 1) < 1e-6
    assert abs(_ke(u, cfg.dx) / row["kinetic_energy"] - 1) < 5e-6


def test_speed_field_N128(golden):
    """runner.py single-device run, sample_config/config_N_128.json."""
    f = golden["speed_fields"][0]
    ref = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", f["file"]))
    cfg = O.OracleConfig(N=128, L=1.0, nu=f["nu"], dt=f["dt"], steps=f["steps"])
    for dtype, tol in ((np.float32, 5e-7), (np.float64, 5e-7)):
        _, u = O.rollout(np.zeros((2, 128, 128), dtype), np.array(f["theta"], dtype), cfg)
        speed = np.sqrt(u[0].astype(np.float64) ** 2 + u[1].astype(np.float64) ** 2)
        assert rel_l2(ref, speed) < tol


def test_speed_field_N512(golden):
    """runner.py 8-device run at N=512 (sample_config/config_N_512.json); the
    distributed result equals the single-device algorithm."""
    f = golden["speed_fields"][1]
    import os
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", f["file"]))
    cfg = O.OracleConfig(N=512, L=1.0, nu=f["nu"], dt=f["dt"], steps=f["steps"])
    _, u = O.rollout(np.zeros((2, 512, 512), np.float32), np.array(f["theta"], np.float32), cfg)
    speed = np.sqrt(u[0].astype(np.float64) ** 2 + u[1].astype(np.float64) ** 2)
    assert rel_l2(ref, speed[::4, ::4]) < 5e-7
    assert abs(np.linalg.norm(speed) / f["full_norm"] - 1) < 5e-7


def test_sgd_trajectory_gradient(golden):
    """The optimisation study's SGD(lr=0.1) steps give the reference's JAX
    gradient: grad(theta_k) = (theta_k - theta_{k+1}) / 0.1.  Central finite
    differences of the float64 oracle reproduce it (B component to the float32
    quantisation of the stored parameters, A to its 5% quantisation)."""
    s = golden["studies"]["sgd"]
    P = np.array(s["parameters"])
    g_ref = (P[0] - P[1]) / s["lr"]
    cfg = O.OracleConfig(N=128, L=1.0, nu=s["nu"], dt=s["dt"], steps=s["steps"], scheme=s["scheme"])
    g = O.fd_gradient(lambda th: O.objective(th, cfg, np.float64), P[0], rel_step=1e-3)
    assert abs(g[1] - g_ref[1]) < 2e-6 + 1e-5 * abs(g_ref[1])
    assert abs(g[0] - g_ref[0]) < 2.5e-6
    assert abs(float(O.objective(P[0], cfg, np.float32)) - s["objectives"][0]) < 1e-7


def test_sgd_objectives_along_trajectory(golden):
    """jit_objective values stored along the SGD trajectory."""
    s = golden["studies"]["sgd"]
    cfg = O.OracleConfig(N=128, L=1.0, nu=s["nu"], dt=s["dt"], steps=s["steps"], scheme=s["scheme"])
    for k in (1, 10, 100):
        th = np.array(s["parameters"][k], np.float32)
        assert abs(float(O.objective(th, cfg, np.float32)) / s["objectives"][k] - 1) < 2e-6


def test_oracle_fp64_close_to_fp32():
    """The float32 and float64 restatements agree on a seeded non-zero IC."""
    from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0
    u0 = spectral_u0(64, 8, 0)
    cfg = O.OracleConfig(N=64, L=2 * math.pi, nu=1e-3, dt=1e-3, steps=20)
    th = np.array([1.0, 0.5], np.float32)
    J32, u32 = O.rollout(u0, th, cfg)
    J64, u64 = O.rollout(u0.astype(np.float64), th.astype(np.float64), cfg)
    assert rel_l2(u64, u32) < 1e-5
    assert abs(J32 / J64 - 1) < 1e-5
