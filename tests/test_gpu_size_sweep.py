"""Every supported grid size against the float32 oracle: a few steps of the
rollout (default launch shapes for each N: tiled stencil at small N, row
bands from N = 1024 on, radix-16 transforms with the smaller final pass where
log2 N is not a multiple of 4), both advection schemes, seeded non-zero
state, on [0, L]^2 with L = 1 and 2 pi."""
import math

import numpy as np
import pytest
import torch

from oracle import ns_oracle as O
from tests.conftest import rel_l2
from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nsgb(cuda_lib):
    import ns_solver_jax_differential_distributed_gb300 as m
    return m


@pytest.mark.parametrize("N", [16, 32, 64, 128, 256, 512, 1024, 2048])
@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_rollout_every_size(nsgb, N, scheme):
    L = 1.0 if N in (32, 512, 2048) else 2 * math.pi
    steps = 5
    dx = L / N
    nu = 1e-3
    dt = float(np.float32(min(0.2 * dx, dx * dx / (8 * nu))))  # well inside both stability limits
    u0 = spectral_u0(N, min(8, N // 4), N)
    th = np.array([0.9, 0.45, nu], np.float32)
    grid = nsgb.make_grid(N, L)
    phys = nsgb.Phys(nu=nu, mu0=0.5, sigma0=0.1, C=1.0)
    s = nsgb.SingleCoreNSSolver(grid, phys, nsgb.Time(dt=dt, steps=steps), scheme)
    J, u = s.rollout(torch.from_numpy(u0).cuda(), torch.from_numpy(th).cuda())
    J32, u32 = O.rollout(u0, th, O.OracleConfig(N=N, L=L, nu=nu, dt=dt, steps=steps, scheme=scheme))
    err = rel_l2(u32, u.cpu().numpy())
    assert err < 1e-5, (N, scheme, err)
    assert abs(float(J) - float(J32)) <= 1e-5 * abs(float(J32)) + 1e-9, (float(J), float(J32))
