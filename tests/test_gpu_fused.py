"""The fused row kernel (inverse row FFT, stencil and forward row FFT in one
launch, with a two-CTA cluster splitting each row at N = 4096) gives the same
bits as the four-kernel step: every row pair is transformed by the same
radix-16 arithmetic and every cell by the same stencil expressions.  Compared
against the four-kernel rollout with the row-streaming stencil of the same
band and radix-16 row passes (which also fixes the grouping of the objective
partials, so J is compared bit for bit too), eager and graph-chunked, both
schemes, full-height and uneven bands; against the float32 oracle at N=1024."""
import math

import numpy as np
import pytest
import torch

from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0

pytestmark = pytest.mark.gpu

L = 2 * math.pi
NU = 1e-3
SCHEMES = {"central": 0, "upwind": 1}


@pytest.fixture(scope="module")
def nat(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    return _native


def _dt(N):
    # CFL-stable for both schemes at every N tested (|u| up to ~3, dx = 2 pi / N)
    return 0.4 / N


def _inputs(N, seed=5):
    u0 = torch.from_numpy(spectral_u0(N, min(32, N // 4), seed)).cuda()
    th = torch.tensor([0.9, 0.4, 2e-3], dtype=torch.float32, device="cuda")
    return u0, th


def _run(nat, N, scheme, steps, use_graph, fused_rows, band_rows):
    """Rollout with the fused kernel (fused_rows > 0) or the four-kernel step
    with the matching band; the plan's settings are restored afterwards."""
    plan = nat.get_plan(N, L, torch.device("cuda"))
    tiles, radix, fused = plan.tiles(), plan.fft_radix(), plan.fused_rows()
    u0, theta = _inputs(N)
    try:
        plan.set_fft_radix(16, radix[1])
        plan.set_tiles(min(N, 2048), band_rows, tiles[2], tiles[3])
        plan.set_fused(fused_rows)
        J, u = nat.op_rollout(u0, theta, steps, L, NU, _dt(N), SCHEMES[scheme], 0.5, 0.1, 1.0, use_graph)
        torch.cuda.synchronize()
        return J.clone(), u.clone()
    finally:
        plan.set_fused(fused)
        plan.set_tiles(*tiles)
        plan.set_fft_radix(*radix)


@pytest.mark.parametrize("scheme", ["central", "upwind"])
@pytest.mark.parametrize("N,rows", [(1024, 14), (2048, 28), (4096, 54), (4096, 4096), (4096, 2), (1024, 1024)])
def test_fused_rollout_bitwise(nat, scheme, N, rows):
    for steps, use_graph in ((1, False), (2, False), (3, False), (40, True)):
        if rows > 512 and steps > 3:
            continue  # few CTAs: slow, and the short cases cover the band logic
        Jf, uf = _run(nat, N, scheme, steps, use_graph, rows, rows)
        Jr, ur = _run(nat, N, scheme, steps, use_graph, 0, rows)
        assert torch.isfinite(ur).all() and math.isfinite(float(Jr)), (steps, use_graph)
        assert torch.equal(uf, ur), (steps, use_graph, (uf - ur).abs().max().item())
        assert torch.equal(Jf, Jr), (steps, use_graph, float(Jf), float(Jr))


def test_fused_default_band_and_stage_timing(nat):
    N = 4096
    plan = nat.get_plan(N, L, torch.device("cuda"))
    old = plan.fused_rows()
    try:
        plan.set_fused(-1)
        rows = plan.fused_rows()
        assert rows > 0 and rows % 2 == 0
        u0, th = _inputs(N)
        st = nat.time_step_pipeline(u0, th, L, NU, _dt(N), "central", steps=4)
        assert set(st) == {"fused", "cols"} and all(v > 0 for v in st.values()), st
    finally:
        plan.set_fused(old)


def test_fused_rejects_bad_bands(nat):
    plan = nat.get_plan(1024, L, torch.device("cuda"))
    with pytest.raises(nat.NativeError):
        plan.set_fused(7)
    with pytest.raises(nat.NativeError):
        nat.get_plan(512, L, torch.device("cuda")).set_fused(16)
    assert plan.fused_rows() == 0


def test_fused_matches_oracle(nat):
    from oracle import ns_oracle as O
    N, steps = 1024, 6
    u0, th = _inputs(N)
    Jf, uf = _run(nat, N, "central", steps, False, 14, 14)
    cfg = O.OracleConfig(N=N, L=L, nu=NU, dt=_dt(N), steps=steps, scheme="central")
    J32, u32 = O.rollout(u0.cpu().numpy(), th.cpu().numpy(), cfg)
    assert O.rel_l2(u32, uf.cpu().numpy()) < 1e-5
    assert abs(float(Jf) - float(J32)) <= 1e-5 * abs(float(J32))
