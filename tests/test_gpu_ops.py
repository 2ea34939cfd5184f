"""GPU parity of the single operators (PeriodicDifferentialOps, advection
schemes, SpectralPoissonSolver, forcing, ChorinProjector.step) against the
float32 oracle.  The stencils keep the reference's operation order without FMA
contraction, so they are compared bit for bit."""
import math

import numpy as np
import pytest
import torch

from oracle import ns_oracle as O
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

SIZES = [16, 64, 256]


def _field(N, seed, comps=0):
    rng = np.random.default_rng(seed)
    shape = (comps, N, N) if comps else (N, N)
    return rng.standard_normal(shape).astype(np.float32)


@pytest.fixture(scope="module")
def nsgb(cuda_lib):
    import ns_solver_jax_differential_distributed_gb300 as m
    return m


@pytest.mark.parametrize("N", SIZES)
@pytest.mark.parametrize("L", [1.0, 2 * math.pi])
def test_stencils_bit_exact(nsgb, N, L):
    dx = L / N
    ops = nsgb.PeriodicDifferentialOps(dx)
    f, ux, uy = _field(N, 1), _field(N, 2), _field(N, 3)
    ux[0, :5] = 0.0  # exercise the u >= 0 branch at zero
    tf, tux, tuy = (torch.from_numpy(a).cuda() for a in (f, ux, uy))
    gx, gy = ops.grad(tf)
    ogx, ogy = O.grad(f, dx)
    assert np.array_equal(gx.cpu().numpy(), ogx) and np.array_equal(gy.cpu().numpy(), ogy)
    assert np.array_equal(ops.laplacian(tf).cpu().numpy(), O.laplacian(f, dx))
    assert np.array_equal(ops.upwind_advect(tf, tux, tuy).cpu().numpy(), O.upwind_advect(f, ux, uy, dx))
    ca = nsgb.CentralAdvection().advect(tf, tux, tuy, ops)
    assert np.array_equal(ca.cpu().numpy(), O.central_advect(f, ux, uy, dx))
    u = np.stack([ux, uy])
    assert np.array_equal(ops.divergence(torch.from_numpy(u).cuda()).cpu().numpy(), O.divergence(u, dx))


@pytest.mark.parametrize("N", [16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192])
def test_poisson_matches_oracle(nsgb, N):
    dx = 2 * math.pi / N
    rhs = _field(N, N)
    p = nsgb.SpectralPoissonSolver(N, N, dx)(torch.from_numpy(rhs).cuda()).cpu().numpy()
    ref64 = O.poisson_solve(rhs.astype(np.float64), dx)
    ref32 = O.poisson_solve(rhs, dx)
    err = rel_l2(ref64, p)
    assert err < 2e-6 * max(1.0, math.log2(N) / 4), err
    assert rel_l2(ref64, ref32) < 2e-6 * max(1.0, math.log2(N) / 4)


def test_poisson_zero_mean_and_linearity(nsgb):
    N = 128
    dx = 1.0 / N
    solver = nsgb.SpectralPoissonSolver(N, N, dx)
    a, b = (torch.from_numpy(_field(N, s)).cuda() for s in (5, 6))
    pa, pb, pab = solver(a), solver(b), solver(2.0 * a + b)
    assert abs(float(pa.double().mean())) < 1e-6
    assert rel_l2((2 * pa + pb).cpu().numpy(), pab.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("N", [16, 128])
def test_forcing_field(nsgb, N):
    grid = nsgb.make_grid(N, 2 * math.pi)
    phys = nsgb.Phys(nu=1e-3, mu0=0.5, sigma0=0.1, C=1.0)
    ff = nsgb.GaussianForcingField(grid, phys)
    th = np.array([0.9, 0.4], np.float32)
    cfg = O.OracleConfig(N=N, L=2 * math.pi, nu=1e-3, dt=1e-3, steps=1)
    for t in (0.0, 0.013, 0.37):
        f = ff(torch.from_numpy(th).cuda(), t).cpu().numpy()
        ref = O.full_forcing(th, np.float32(t), cfg)
        assert f.shape == (2, N, N) and np.all(f[1] == 0)
        np.testing.assert_allclose(f, ref, rtol=2e-6, atol=1e-7)


@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_projector_step_generic_force(nsgb, scheme):
    N, L = 64, 2 * math.pi
    dx, dt, nu = L / N, 1e-3, 2e-3
    from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0
    u = spectral_u0(N, 8, 2)
    f = _field(N, 9, comps=2)
    proj = nsgb.ChorinProjector(nsgb.PeriodicDifferentialOps(dx), nsgb.SpectralPoissonSolver(N, N, dx),
                                nsgb.make_advection_scheme(scheme), nu, dt)
    out = proj.step(torch.from_numpy(u).cuda(), torch.from_numpy(f).cuda()).cpu().numpy()
    cfg = O.OracleConfig(N=N, L=L, nu=nu, dt=dt, steps=1, scheme=scheme)
    ref = O.projector_step(u, f, cfg)
    assert rel_l2(ref, out) < 1e-6


def test_generic_strategy_composition(nsgb):
    """A user-defined DifferentialOps subclass falls back to the reference's
    composition of its own methods (each still a CUDA op)."""
    N, L = 32, 1.0
    dx = L / N

    class MyOps(nsgb.PeriodicDifferentialOps):
        pass

    from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0
    u = spectral_u0(N, 4, 1)
    f = _field(N, 4, comps=2)
    a = nsgb.ChorinProjector(MyOps(dx), nsgb.SpectralPoissonSolver(N, N, dx), nsgb.UpwindAdvection(), 1e-2, 1e-3)
    b = nsgb.ChorinProjector(nsgb.PeriodicDifferentialOps(dx), nsgb.SpectralPoissonSolver(N, N, dx),
                             nsgb.UpwindAdvection(), 1e-2, 1e-3)
    ua = a.step(torch.from_numpy(u).cuda(), torch.from_numpy(f).cuda()).cpu().numpy()
    ub = b.step(torch.from_numpy(u).cuda(), torch.from_numpy(f).cuda()).cpu().numpy()
    assert rel_l2(ub, ua) < 1e-6


def test_cpu_tensor_rejected(nsgb):
    ops = nsgb.PeriodicDifferentialOps(0.1)
    with pytest.raises(Exception):
        ops.laplacian(torch.zeros(16, 16))
