"""The FFT-Poisson solve in radix 8 (row and/or column passes) agrees with
the radix-16 solve and with the oracle's spectral solve to FFT rounding, and a
rollout with radix-8 passes keeps the parity bars against the float32 oracle."""
import math

import numpy as np
import pytest
import torch

from oracle import ns_oracle as O
from tests.conftest import rel_l2
from ns_solver_jax_differential_distributed_gb300.workloads import PLAIN_SMALL

pytestmark = pytest.mark.gpu

L = 2 * math.pi


@pytest.fixture(scope="module")
def nat(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    return _native


def _with_radix(nat, N, radix, fn, rows=None):
    plan = nat.get_plan(N, L, torch.device("cuda"))
    old_r, old_t = plan.fft_radix(), plan.tiles()
    if rows is not None:
        plan.set_tiles(old_t[0], old_t[1], rows, old_t[3])
    plan.set_fft_radix(*radix)
    try:
        out = fn()
        torch.cuda.synchronize()
        return out
    finally:
        plan.set_fft_radix(*old_r)
        plan.set_tiles(*old_t)


@pytest.mark.parametrize("N", [16, 32, 64, 256, 1024, 4096, 8192])
def test_poisson_radix8_matches_radix16_and_oracle(nat, N):
    rng = np.random.default_rng(N)
    rhs = rng.standard_normal((N, N)).astype(np.float32)
    rhs -= rhs.mean(dtype=np.float64).astype(np.float32)
    t = torch.from_numpy(rhs).cuda()
    p16 = _with_radix(nat, N, (16, 16), lambda: nat.op_poisson(t, L).clone())
    ref = O.poisson_solve(rhs.astype(np.float64), L / N)
    radices, rows = ((8, 8), (8, 16), (16, 8)), None
    if N == 8192:
        # a radix-8 transform of 8192 takes 1024 threads: the column kernel
        # allows 512 and the row kernels one row pair per CTA, so the plan
        # refuses the radix-8 column pass and radix-8 rows need 2 rows per CTA
        for bad in ((8, 8), (16, 8)):
            with pytest.raises(nat.NativeError):
                _with_radix(nat, N, bad, lambda: None, rows=2)
        with pytest.raises(nat.NativeError):
            _with_radix(nat, N, (8, 16), lambda: None, rows=4)
        radices, rows = ((8, 16),), 2
    for radix in radices:
        p = _with_radix(nat, N, radix, lambda: nat.op_poisson(t, L).clone(), rows=rows)
        assert rel_l2(p16.double().cpu().numpy(), p.double().cpu().numpy()) < 2e-6, radix
        assert rel_l2(ref, p.double().cpu().numpy()) < 5e-6, radix


@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_rollout_radix8_parity(nat, scheme):
    w = PLAIN_SMALL
    u0, th = w.u0(), w.theta()
    sch = {"central": 0, "upwind": 1}[scheme]
    for steps, tol in ((1, 1e-5), (100, 1e-4)):
        def run():
            J, u = nat.op_rollout(torch.from_numpy(u0).cuda(), torch.from_numpy(th).cuda(), steps, w.L, w.nu,
                                  w.dt, sch, 0.5, 0.1, 1.0, True)
            return J.clone(), u.clone()
        J, u = _with_radix(nat, w.N, (8, 8), run)
        cfg = O.OracleConfig(N=w.N, L=w.L, nu=w.nu, dt=w.dt, steps=steps, scheme=scheme)
        J32, u32 = O.rollout(u0, th, cfg)
        assert rel_l2(u32, u.cpu().numpy()) < tol, (steps, rel_l2(u32, u.cpu().numpy()))
        assert abs(float(J) - float(J32)) <= tol * abs(float(J32)) + 1e-9


def test_radix_validation(nat):
    plan = nat.get_plan(64, L, torch.device("cuda"))
    r = plan.fft_radix()
    with pytest.raises(nat.NativeError):
        plan.set_fft_radix(4, 16)
    assert plan.fft_radix() == r
