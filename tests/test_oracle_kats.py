"""The reference's single-device known-answer tests, applied to the oracle
(unit_tests/test_distributed_solver.py:258-416)."""
import numpy as np

from oracle import ns_oracle as O


def _max_div(u, dx):
    gx = (np.roll(u[0], -1, 0) - np.roll(u[0], 1, 0)) / (2 * dx)
    gy = (np.roll(u[1], -1, 1) - np.roll(u[1], 1, 1)) / (2 * dx)
    return float(np.max(np.abs(gx + gy)))


def test_step_divergence_free():
    cfg = O.OracleConfig(N=32, L=1.0, nu=0.01, dt=0.001, steps=1)
    u1 = O.solver_step(np.zeros((2, 32, 32), np.float32), np.array([0.9, 0.4], np.float32), 0.0, cfg)
    assert _max_div(u1, cfg.dx) < 5e-4


def test_rollout_divergence_free():
    cfg = O.OracleConfig(N=32, L=1.0, nu=0.01, dt=0.001, steps=5)
    _, u = O.rollout(np.zeros((2, 32, 32), np.float32), np.array([0.9, 0.4], np.float32), cfg)
    assert _max_div(u, cfg.dx) < 1e-3


def _lap_err(N):
    dx = 1.0 / N
    x = np.linspace(0.0, 1.0, N, endpoint=False)
    X, Y = np.meshgrid(x, x, indexing="ij")
    u = np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y)
    return float(np.max(np.abs(O.laplacian(u, dx) + 2 * (2 * np.pi) ** 2 * u)))


def test_laplacian_second_order():
    e16, e32, e64 = _lap_err(16), _lap_err(32), _lap_err(64)
    assert e16 / e32 > 3.5 and e32 / e64 > 3.5


def test_poisson_manufactured_and_monotone():
    errs = {}
    for N in (32, 64):
        dx = 1.0 / N
        x = np.linspace(0.0, 1.0, N, endpoint=False)
        X, Y = np.meshgrid(x, x, indexing="ij")
        p_exact = np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y)
        rhs = (-2 * (2 * np.pi) ** 2 * p_exact).astype(np.float32)
        errs[N] = float(np.max(np.abs(O.poisson_solve(rhs, dx) - p_exact)))
        assert errs[N] < 2e-4
    assert errs[64] <= errs[32] + 1e-6


def test_unknown_scheme_raises():
    import pytest
    with pytest.raises(ValueError):
        O.advect(np.zeros((4, 4)), np.zeros((4, 4)), np.zeros((4, 4)), 0.1, "quick")
