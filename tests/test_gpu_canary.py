"""Canary-guarded buffers: every output and workspace an entry point writes is
placed between two 64 KiB guard regions filled with a byte pattern, and after
the call the guards must be intact (and inputs unchanged).  compute-sanitizer
is closed on this machine; this catches writes past either end of a buffer --
the row-band halos, the periodic wraps, the FFT staging and the objective
partials -- on the kernels' real launch shapes, through the C ABI.  Covered:
the single operators, the Poisson solve (plan and no-allocation forms), a
solver step, rollouts (tiled and row-streaming stencils, column bands with
halo groups at N=4096, graph chunks, the fused row kernel), the checkpointed
gradient and a batched ensemble."""
import ctypes
import math

import numpy as np
import pytest
import torch

from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0

pytestmark = pytest.mark.gpu

GUARD = 1 << 16
CANARY = 0xA5
L = 2 * math.pi


@pytest.fixture(scope="module")
def nat(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    return _native


class Guarded:
    """A device buffer of `nbytes` (256-byte aligned) between two guards."""

    def __init__(self, nbytes: int, fill=None):
        self.nbytes = int(nbytes)
        self.raw = torch.full((2 * GUARD + self.nbytes,), CANARY, dtype=torch.uint8, device="cuda")
        self.inner = self.raw[GUARD:GUARD + self.nbytes]
        if fill is not None:
            self.inner.copy_(fill.contiguous().view(torch.uint8).reshape(-1))

    def f32(self, *shape):
        return self.inner.view(torch.float32).view(*shape)

    def ptr(self):
        return self.inner.data_ptr()

    def intact(self) -> bool:
        torch.cuda.synchronize()
        return bool((self.raw[:GUARD] == CANARY).all()) and bool((self.raw[GUARD + self.nbytes:] == CANARY).all())


def _fields(N, seed=2):
    u0 = torch.from_numpy(spectral_u0(N, min(8, N // 4), seed)).cuda()
    th = torch.tensor([0.9, 0.4, 2e-3], dtype=torch.float32, device="cuda")
    return u0, th


def _phys(nat, scheme, dt=1e-3, nu=2e-3):
    return nat.make_phys(L, nu, dt, scheme)


@pytest.mark.parametrize("N", [64, 1024])
def test_single_operators_and_poisson(nat, N):
    lib = nat.lib()
    plan = nat.get_plan(N, L, torch.device("cuda"))
    st = torch.cuda.current_stream().cuda_stream
    u0, _ = _fields(N)
    f = u0[0].contiguous()
    nb = 4 * N * N
    outs = [Guarded(nb) for _ in range(3)]
    assert lib.nsgb_grad(plan.handle, f.data_ptr(), outs[0].ptr(), outs[1].ptr(), st) == 0
    assert lib.nsgb_laplacian(plan.handle, f.data_ptr(), outs[2].ptr(), st) == 0
    div = Guarded(nb)
    assert lib.nsgb_divergence(plan.handle, u0.data_ptr(), div.ptr(), st) == 0
    adv = [Guarded(nb) for _ in range(2)]
    for k, sid in enumerate((0, 1)):
        assert lib.nsgb_advect(plan.handle, sid, f.data_ptr(), u0[0].data_ptr(), u0[1].data_ptr(),
                               adv[k].ptr(), st) == 0
    ws = Guarded(lib.nsgb_poisson_workspace_bytes(plan.handle))
    p = Guarded(nb)
    assert lib.nsgb_poisson(plan.handle, div.ptr(), p.ptr(), ws.ptr(), ws.nbytes, st) == 0
    pn = Guarded(nb)
    if N <= 1024:
        assert lib.nsgb_poisson_noalloc(N, L, div.ptr(), pn.ptr(), st) == 0
    for b in outs + [div, ws, p, pn] + adv:
        assert b.intact()


@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_step_and_projector_step(nat, scheme):
    lib = nat.lib()
    N = 256
    plan = nat.get_plan(N, L, torch.device("cuda"))
    st = torch.cuda.current_stream().cuda_stream
    u0, th = _fields(N)
    keep = u0.clone()
    ph = _phys(nat, scheme)
    ws = Guarded(lib.nsgb_step_workspace_bytes(plan.handle))
    out = Guarded(8 * N * N)
    assert lib.nsgb_step(plan.handle, ctypes.byref(ph), u0.data_ptr(), th.data_ptr(), 3, ctypes.c_float(0.01),
                         out.ptr(), ws.ptr(), ws.nbytes, st) == 0
    force = torch.zeros_like(u0)
    out2 = Guarded(8 * N * N)
    assert lib.nsgb_projector_step(plan.handle, ctypes.byref(ph), u0.data_ptr(), force.data_ptr(), out2.ptr(),
                                   ws.ptr(), ws.nbytes, st) == 0
    assert ws.intact() and out.intact() and out2.intact()
    assert torch.equal(u0, keep)


@pytest.mark.parametrize("N,tiles,fused,steps", [
    (64, (32, 8), 0, 40),            # tiled stencil, graph chunks
    (1024, (256, 24), 0, 5),         # row bands with halo groups
    (1024, (1024, 14), 14, 40),      # fused row kernel, graph chunks
    (4096, (2048, 54), 0, 3),        # the headline band shape
    (4096, (2048, 54), 54, 3),       # fused, two-CTA clusters
])
def test_rollout(nat, N, tiles, fused, steps):
    lib = nat.lib()
    plan = nat.get_plan(N, L, torch.device("cuda"))
    old_t, old_r, old_f = plan.tiles(), plan.fft_radix(), plan.fused_rows()
    st = torch.cuda.current_stream().cuda_stream
    u0, th = _fields(N)
    keep = u0.clone()
    ph = _phys(nat, "upwind", dt=0.4 / N)
    try:
        plan.set_fft_radix(16, 16)
        plan.set_tiles(tiles[0], tiles[1], old_t[2], old_t[3])
        plan.set_fused(fused)
        ws = Guarded(lib.nsgb_rollout_workspace_bytes(plan.handle, steps))
        uf, J = Guarded(8 * N * N), Guarded(256)
        assert lib.nsgb_rollout(plan.handle, ctypes.byref(ph), u0.data_ptr(), th.data_ptr(), 3, steps, uf.ptr(),
                                J.ptr(), ws.ptr(), ws.nbytes, 1, st) == 0, lib.nsgb_last_error()
        assert ws.intact() and uf.intact() and J.intact()
        assert torch.equal(u0, keep) and torch.isfinite(uf.f32(2, N, N)).all()
    finally:
        plan.set_fused(old_f)
        plan.set_tiles(*old_t)
        plan.set_fft_radix(*old_r)


@pytest.mark.parametrize("N", [64, 1024])
def test_gradient(nat, N):
    lib = nat.lib()
    plan = nat.get_plan(N, L, torch.device("cuda"))
    st = torch.cuda.current_stream().cuda_stream
    u0, th = _fields(N)
    ph = _phys(nat, "upwind", dt=0.4 / N)
    steps, every = 9, 4
    ws = Guarded(lib.nsgb_rollout_grad_workspace_bytes(plan.handle, steps, every))
    J, uf, g, du0 = Guarded(256), Guarded(8 * N * N), Guarded(256), Guarded(8 * N * N)
    phases = nat.GRAD_FORWARD | nat.GRAD_BACKWARD
    assert lib.nsgb_rollout_grad(plan.handle, ctypes.byref(ph), u0.data_ptr(), th.data_ptr(), 3, steps, every,
                                 phases, J.ptr(), uf.ptr(), g.ptr(), du0.ptr(), ws.ptr(), ws.nbytes, st) == 0
    for b in (ws, J, uf, g, du0):
        assert b.intact()
    assert np.isfinite(g.f32(64)[:3].cpu().numpy()).all()


def test_ensemble(nat):
    lib = nat.lib()
    st = torch.cuda.current_stream().cuda_stream
    sizes = [64, 128, 64, 256]
    steps = 20
    arr = (nat.Member * len(sizes))()
    keep = []
    guards = []
    for k, N in enumerate(sizes):
        u0, th = _fields(N, seed=k)
        plan = nat.get_plan(N, L, torch.device("cuda"))
        uf, J = Guarded(8 * N * N), Guarded(256)
        keep += [u0, th, plan]
        guards += [uf, J]
        arr[k].plan = plan.handle.value
        arr[k].phys = _phys(nat, "central")
        arr[k].u0 = u0.data_ptr()
        arr[k].theta = th.data_ptr()
        arr[k].theta_len = 3
        arr[k].u_final = uf.ptr()
        arr[k].J = J.ptr()
        arr[k].state = None
        arr[k].total_steps = steps
        arr[k].done_steps = 0
    ws = Guarded(lib.nsgb_ensemble_workspace_bytes(arr, len(sizes)))
    assert lib.nsgb_ensemble_rollout(arr, len(sizes), 8, ws.ptr(), ws.nbytes, st) == 0, lib.nsgb_last_error()
    assert ws.intact() and all(b.intact() for b in guards)
