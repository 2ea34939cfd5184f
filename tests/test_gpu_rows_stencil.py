"""The row-streaming stencil (launch shapes with a band width >= 256) gives
the same bits as the tiled stencil: both evaluate the same per-cell
expressions and differ only in how the grid is split.  Covered: whole rows
(band width = N, periodic wrap inside a CTA), column bands with halo groups
(width < N), uneven row bands, the first step (no pending projection), graph
chunks, the checkpointed gradient path and batched ensembles.  The objective
J sums per-block partials, so it agrees to rounding only."""
import math

import numpy as np
import pytest
import torch

from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0

pytestmark = pytest.mark.gpu

L = 2 * math.pi
NU, DT = 1e-3, 1e-3
SCHEMES = {"central": 0, "upwind": 1}


@pytest.fixture(scope="module")
def nat(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    return _native


def _with_tiles(nat, N, tiles, fn):
    plan = nat.get_plan(N, L, torch.device("cuda"))
    old = plan.tiles()
    plan.set_tiles(*tiles)
    try:
        out = fn()
        torch.cuda.synchronize()
        return out
    finally:
        plan.set_tiles(*old)


def _inputs(N, seed=3):
    u0 = torch.from_numpy(spectral_u0(N, min(8, N // 4), seed)).cuda()
    th = torch.tensor([0.9, 0.4, 2e-3], dtype=torch.float32, device="cuda")
    return u0, th


@pytest.mark.parametrize("scheme", ["central", "upwind"])
@pytest.mark.parametrize("N,tw,th", [(64, 256, 64), (64, 256, 7), (256, 256, 16), (512, 256, 13),
                                     (1024, 512, 64), (1024, 256, 5), (2048, 2048, 31)])
def test_rows_rollout_bitwise(nat, scheme, N, tw, th):
    u0, theta = _inputs(N)
    steps = 20
    for use_graph in (False, True):
        def run():
            J, u = nat.op_rollout(u0, theta, steps, L, NU, DT, SCHEMES[scheme], 0.5, 0.1, 1.0, use_graph)
            return J.clone(), u.clone()
        base = nat.get_plan(N, L, torch.device("cuda")).tiles()
        J_t, u_t = run()
        J_r, u_r = _with_tiles(nat, N, (tw, th, base[2], base[3]), run)
        assert torch.equal(u_t, u_r), (use_graph, (u_t - u_r).abs().max().item())
        assert abs(float(J_t) - float(J_r)) <= 1e-6 * abs(float(J_t)) + 1e-12


@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_rows_gradient_bitwise(nat, scheme):
    N = 256
    u0, theta = _inputs(N, 5)

    def run():
        J, g, uf, du0 = nat.rollout_grad_raw(u0, theta, 12, 5, L, NU, DT, SCHEMES[scheme], want_du0=True,
                                             own_workspace=True)
        return J.clone(), g.clone(), uf.clone(), du0.clone()
    base = nat.get_plan(N, L, torch.device("cuda")).tiles()
    J_t, g_t, uf_t, du_t = run()
    J_r, g_r, uf_r, du_r = _with_tiles(nat, N, (256, 11, base[2], base[3]), run)
    assert torch.equal(uf_t, uf_r)
    assert torch.equal(du_t, du_r)
    assert torch.equal(g_t, g_r)
    assert abs(float(J_t) - float(J_r)) <= 1e-6 * abs(float(J_t)) + 1e-12


def test_rows_ensemble_bitwise(nat):
    from ns_solver_jax_differential_distributed_gb300 import ensemble as E
    from ns_solver_jax_differential_distributed_gb300.workloads import ensemble as make_ensemble
    members = make_ensemble(count=10, steps=1, sizes=(32, 64, 128), probs=(0.3, 0.4, 0.3), seed=11)
    specs = E.from_workload(members)
    J_t, us_t = E.Ensemble(specs, steps=23, chunk=8).run()
    J_t = J_t.clone()
    us_t = [u.clone() for u in us_t]
    plans = {N: nat.get_plan(N, L, torch.device("cuda")) for N in (32, 64, 128)}
    old = {N: p.tiles() for N, p in plans.items()}
    try:
        for N, p in plans.items():
            p.set_tiles(256, 9 if N > 32 else N, old[N][2], old[N][3])
        J_r, us_r = E.Ensemble(specs, steps=23, chunk=8).run()
        torch.cuda.synchronize()
    finally:
        for N, p in plans.items():
            p.set_tiles(*old[N])
    for a, b in zip(us_t, us_r):
        assert torch.equal(a, b)
    # float32 block partials summed over different blocks: rounding-level
    rel = ((J_t.double() - J_r.double()).abs() / J_t.double().abs().clamp_min(1e-30)).max().item()
    assert rel < 1e-5, rel


def test_rows_shape_validation(nat):
    plan = nat.get_plan(64, L, torch.device("cuda"))
    base = plan.tiles()
    with pytest.raises(nat.NativeError):
        plan.set_tiles(384, 8, base[2], base[3])    # band width not a power of two
    with pytest.raises(nat.NativeError):
        plan.set_tiles(4096, 8, base[2], base[3])   # wider than the kernel's block
    with pytest.raises(nat.NativeError):
        plan.set_tiles(256, 65, base[2], base[3])   # more rows than N
    assert plan.tiles() == base
