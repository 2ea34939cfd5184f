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


# Advection: the reference's shipped outputs never exercise it (zero initial
# states), so these known answers pin the oracle's advection operators
# (NS_solver.py:243-247, 257-265, 474-477): -(u.grad)f with x along axis 0,
# central differences, and one-sided upwind differences taken from the side
# the velocity comes from (backward for u >= 0, forward for u < 0).
def _wave(N, m, axis):
    x = np.arange(N, dtype=np.float64) / N
    w = np.sin(2 * np.pi * m * x)
    return np.broadcast_to(w[:, None] if axis == 0 else w[None, :], (N, N)).copy()


def test_central_advection_known_answer_and_order():
    errs = []
    for N in (32, 64, 128):
        h, m, c = 1.0 / N, 3, 0.7
        x = np.arange(N) / N
        for axis in (0, 1):
            f = _wave(N, m, axis)
            vel = np.full((N, N), c)
            zero = np.zeros((N, N))
            ux, uy = (vel, zero) if axis == 0 else (zero, vel)
            exact_discrete = -c * np.cos(2 * np.pi * m * x) * np.sin(2 * np.pi * m * h) / h
            exact_discrete = exact_discrete[:, None] if axis == 0 else exact_discrete[None, :]
            assert np.max(np.abs(O.central_advect(f, ux, uy, h) - exact_discrete)) < 1e-9
        cont = -c * 2 * np.pi * m * np.cos(2 * np.pi * m * x)[:, None]
        errs.append(np.max(np.abs(O.central_advect(_wave(N, m, 0), np.full((N, N), c), np.zeros((N, N)), h) - cont)))
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5  # second order


def test_upwind_advection_known_answer_sides_and_order():
    errs = []
    for N in (32, 64, 128):
        h, m = 1.0 / N, 2
        x = np.arange(N) / N
        s = 2 * np.pi * m
        backward = (np.sin(s * x) - np.sin(s * (x - h))) / h   # f - f(x - h): velocity >= 0
        forward = (np.sin(s * (x + h)) - np.sin(s * x)) / h    # f(x + h) - f: velocity < 0
        for axis in (0, 1):
            f = _wave(N, m, axis)
            zero = np.zeros((N, N))
            for c, diff in ((0.7, backward), (-0.7, forward)):
                vel = np.full((N, N), c)
                ux, uy = (vel, zero) if axis == 0 else (zero, vel)
                want = -c * (diff[:, None] if axis == 0 else diff[None, :])
                assert np.max(np.abs(O.upwind_advect(f, ux, uy, h) - want)) < 1e-9
        cont = -0.7 * s * np.cos(s * x)[:, None]
        errs.append(np.max(np.abs(O.upwind_advect(_wave(N, m, 0), np.full((N, N), 0.7), np.zeros((N, N)), h)
                                  - cont)))
    assert 1.8 < errs[0] / errs[1] < 2.2 and 1.8 < errs[1] / errs[2] < 2.2  # first order


def test_upwind_side_switches_per_cell():
    """Mixed signs in one field: each cell takes its own side (u = 0 counts
    as non-negative, the reference's >=)."""
    N, h = 16, 1.0 / 16
    rng = np.random.default_rng(5)
    f = rng.standard_normal((N, N))
    ux = rng.choice([-1.0, 0.0, 1.0], size=(N, N))
    uy = np.zeros((N, N))
    got = O.upwind_advect(f, ux, uy, h)
    for i in range(N):
        for j in range(N):
            d = (f[i, j] - f[i - 1, j]) if ux[i, j] >= 0 else (f[(i + 1) % N, j] - f[i, j])
            assert abs(got[i, j] + ux[i, j] * d / h) < 1e-9
