"""Batched gradient solves (nsgb_grad_batch_advance): every solve's J,
dJ/dtheta and dJ/du0 equal its own nsgb_rollout_grad bit for bit, for mixed
N, schemes, step counts and checkpoint intervals, work split into uneven
slices, and solves that join a batch already in progress."""
import ctypes
import math

import pytest
import torch

from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0

pytestmark = pytest.mark.gpu

L = 2 * math.pi


@pytest.fixture(scope="module")
def mods(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native, ensemble
    return _native, ensemble


def _case(N, seed):
    u0 = torch.from_numpy(spectral_u0(N, min(8, N // 4), seed)).cuda()
    th = torch.tensor([0.9 + 0.01 * seed, 0.4, 2e-3], dtype=torch.float32, device="cuda")
    return u0, th


CASES = [  # N, scheme, steps, every
    (32, "central", 1, 1),
    (32, "upwind", 9, 4),
    (64, "central", 13, 5),
    (64, "central", 7, 50),
    (64, "upwind", 70, 8),      # more than 64 adjoint steps: a mid-sweep partial reduction
    (128, "upwind", 5, 1),
    (128, "central", 6, 3),
    (1024, "upwind", 3, 2),     # row-streaming forward and adjoint kernels
]


def _reference(_native, u0, th, N, scheme, steps, every, want_du0=False):
    dt = 0.4 / N
    J, g, _, du0 = _native.rollout_grad_raw(u0, th, steps, every, L, 1e-3, dt, scheme, want_u_final=False,
                                            want_du0=want_du0, own_workspace=True)
    return J.clone(), g.clone(), (du0.clone() if want_du0 else None)


def test_batch_equals_single_calls(mods):
    _native, ensemble = mods
    refs, ids = [], []
    gb = ensemble.GradientBatch()
    late = len(CASES) - 2  # the last two join after the first slice
    for k, (N, scheme, steps, every) in enumerate(CASES):
        u0, th = _case(N, k)
        refs.append(_reference(_native, u0, th, N, scheme, steps, every, want_du0=(k == 2)))
        if k < late:
            ids.append(gb.add(u0, th, steps, every, L, 1e-3, 0.4 / N, scheme, want_du0=(k == 2)))
    gb.advance(7)
    for k in range(late, len(CASES)):
        N, scheme, steps, every = CASES[k]
        u0, th = _case(N, k)
        ids.append(gb.add(u0, th, steps, every, L, 1e-3, 0.4 / N, scheme))
    calls = 1
    while gb.pending():
        gb.advance(11)
        calls += 1
    torch.cuda.synchronize()
    assert calls > 3
    for k, sid in enumerate(ids):
        J, g = gb.result(sid)
        Jr, gr, dur = refs[k]
        assert torch.isfinite(g).all()
        assert torch.equal(J, Jr), (k, float(J), float(Jr))
        assert torch.equal(g, gr), (k, g.tolist(), gr.tolist())
        if dur is not None:
            assert torch.equal(gb.du0(sid), dur)


def test_one_call_and_single_op_slices_agree(mods):
    _native, ensemble = mods
    N, scheme, steps, every = 64, "upwind", 6, 4
    u0, th = _case(N, 3)
    a, b = ensemble.GradientBatch(), ensemble.GradientBatch()
    ia = a.add(u0, th, steps, every, L, 1e-3, 0.4 / N, scheme)
    ib = b.add(u0, th, steps, every, L, 1e-3, 0.4 / N, scheme)
    total = _native.lib().nsgb_grad_ops(steps, every)
    assert total == steps + 2 * 4 + 2 * 2  # segments of 4 and 2 steps: recompute + adjoint each
    assert a.advance(total) == [ia]
    n = 0
    while b.pending():
        b.advance(1)
        n += 1
    assert n == total
    torch.cuda.synchronize()
    assert torch.equal(a.result(ia)[0], b.result(ib)[0]) and torch.equal(a.result(ia)[1], b.result(ib)[1])


def test_refuses_capturing_stream(mods):
    _native, ensemble = mods
    N = 32
    u0, th = _case(N, 0)
    gb = ensemble.GradientBatch()
    sid = gb.add(u0, th, 3, 2, L, 1e-3, 0.4 / N, "central")
    rec = gb._solves[sid]
    lib = _native.lib()
    arr = (_native.GradMember * 1)(rec["member"])
    need = lib.nsgb_grad_batch_workspace_bytes(1, 4)
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            rc = lib.nsgb_grad_batch_advance(arr, 1, 4, ws.data_ptr(), ws.numel(), ctypes.c_void_p(s.cuda_stream))
        finally:
            g.capture_end()
    assert rc == 1 and b"capturing" in lib.nsgb_last_error()


def test_rejects_members_sharing_a_state(mods):
    _native, ensemble = mods
    N = 32
    u0, th = _case(N, 0)
    gb = ensemble.GradientBatch()
    sid = gb.add(u0, th, 3, 2, L, 1e-3, 0.4 / N, "central")
    m = gb._solves[sid]["member"]
    lib = _native.lib()
    arr = (_native.GradMember * 2)(m, m)
    ws = torch.empty(lib.nsgb_grad_batch_workspace_bytes(2, 4), dtype=torch.uint8, device="cuda")
    rc = lib.nsgb_grad_batch_advance(arr, 2, 4, ws.data_ptr(), ws.numel(), _native.stream_of(torch.device("cuda")))
    assert rc == 1 and b"share" in lib.nsgb_last_error()


def test_u_final_and_two_parameter_theta(mods):
    """The final state written at the end of the forward phase, and theta
    [A, B] (nu from the physics), against nsgb_rollout_grad."""
    _native, ensemble = mods
    gb = ensemble.GradientBatch()
    ids, refs = [], []
    for k, (N, scheme, steps, every) in enumerate([(64, "upwind", 11, 3), (128, "central", 4, 4)]):
        u0, th = _case(N, k)
        th2 = th[:2].contiguous()
        J, g, uf, _ = _native.rollout_grad_raw(u0, th2, steps, every, L, 1e-3, 0.4 / N, scheme, want_u_final=True,
                                               own_workspace=True)
        refs.append((J.clone(), g.clone(), uf.clone()))
        ids.append(gb.add(u0, th2, steps, every, L, 1e-3, 0.4 / N, scheme, want_u_final=True))
    gb.run(5)
    torch.cuda.synchronize()
    for sid, (J, g, uf) in zip(ids, refs):
        Jb, gb_ = gb.result(sid)
        assert gb_.numel() == 2
        assert torch.equal(Jb, J) and torch.equal(gb_, g) and torch.equal(gb.u_final(sid), uf)


def test_refuses_bad_solves_and_unfinished_reads(mods):
    """add() refuses a theta of 4 entries, steps or every below 1 and an
    unknown scheme before allocating anything; results of a solve that has
    not finished are refused, and are there once it has."""
    _native, ensemble = mods
    gb = ensemble.GradientBatch()
    u0, th = _case(32, 0)
    with pytest.raises(ValueError, match="theta must have 2 or 3"):
        gb.add(u0, torch.ones(4, device="cuda"), 4, 2, L, 1e-3, 0.01, "central")
    for steps, every in ((0, 1), (4, 0)):
        with pytest.raises(ValueError, match="must be >= 1"):
            gb.add(u0, th, steps, every, L, 1e-3, 0.01, "central")
    with pytest.raises(ValueError, match="Unknown advection scheme"):
        gb.add(u0, th, 4, 2, L, 1e-3, 0.01, "lax")
    assert gb.pending() == []
    sid = gb.add(u0, th, 4, 2, L, 1e-3, 0.4 / 32, "central", want_du0=True, want_u_final=True)
    gb.advance(3)
    for read in (gb.result, gb.du0, gb.u_final):
        with pytest.raises(RuntimeError, match="has done 3 of its"):
            read(sid)
    gb.run(5)
    J, g = gb.result(sid)
    Jr, gr, _ = _reference(_native, u0, th, 32, "central", 4, 2)
    assert torch.equal(J, Jr) and torch.equal(g, gr)
