"""The reference's single-device known-answer tests run through the GPU
solver (unit_tests/test_distributed_solver.py:258-416)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nsgb(cuda_lib):
    import ns_solver_jax_differential_distributed_gb300 as m
    return m


def _max_div(u, dx):
    gx = (np.roll(u[0], -1, axis=0) - np.roll(u[0], 1, axis=0)) / (2.0 * dx)
    gy = (np.roll(u[1], -1, axis=1) - np.roll(u[1], 1, axis=1)) / (2.0 * dx)
    return float(np.max(np.abs(gx + gy)))


def _solver(nsgb, steps):
    grid = nsgb.make_grid(32, L=1.0)
    phys = nsgb.Phys(nu=0.01, mu0=0.5, sigma0=0.1, C=1.0)
    return nsgb.SingleCoreNSSolver(grid, phys, nsgb.Time(dt=0.001, steps=steps)), grid


def test_single_core_step_divergence_free(nsgb):
    solver, grid = _solver(nsgb, 1)
    u0 = torch.zeros((2, 32, 32), dtype=torch.float32, device="cuda")
    u1 = solver.step(u0, torch.tensor([0.9, 0.4]), t=0.0).cpu().numpy()
    assert _max_div(u1, grid.dx) < 5e-4


def test_single_core_rollout_final_state_divergence_free(nsgb):
    solver, grid = _solver(nsgb, 5)
    _, u = solver.rollout(torch.zeros((2, 32, 32), device="cuda"), torch.tensor([0.9, 0.4]))
    assert _max_div(u.cpu().numpy(), grid.dx) < 1e-3


def _laplacian_error(nsgb, N):
    dx = 1.0 / N
    x = np.linspace(0.0, 1.0, N, endpoint=False)
    X, Y = np.meshgrid(x, x, indexing="ij")
    u = np.sin(2.0 * np.pi * X) * np.cos(2.0 * np.pi * Y)
    lap = nsgb.PeriodicDifferentialOps(dx).laplacian(torch.tensor(u, dtype=torch.float32, device="cuda"))
    return float(np.max(np.abs(lap.double().cpu().numpy() + 2.0 * (2.0 * np.pi) ** 2 * u)))


def test_laplacian_second_order_convergence(nsgb):
    e16, e32, e64 = (_laplacian_error(nsgb, N) for N in (16, 32, 64))
    assert e16 / e32 > 3.5 and e32 / e64 > 3.5


def test_poisson_manufactured_solution_and_monotone(nsgb):
    errors = {}
    for N in (32, 64):
        dx = 1.0 / N
        x = np.linspace(0.0, 1.0, N, endpoint=False)
        X, Y = np.meshgrid(x, x, indexing="ij")
        p_exact = np.sin(2.0 * np.pi * X) * np.cos(2.0 * np.pi * Y)
        rhs = -2.0 * (2.0 * np.pi) ** 2 * p_exact
        p = nsgb.SpectralPoissonSolver(N, N, dx)(torch.tensor(rhs, dtype=torch.float32, device="cuda"))
        errors[N] = float(np.max(np.abs(p.double().cpu().numpy() - p_exact)))
        assert errors[N] < 2e-4
    assert errors[64] <= errors[32] + 1e-6
