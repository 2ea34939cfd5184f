"""The bounds-checking build (libnsgb_checked.so, NSGB_CHECK_BOUNDS): every
global-memory access of every kernel is checked against the valid device
ranges -- the library's own tables and scratch plus the buffers registered
here with their exact sizes -- and an access outside them is skipped and
reported as NSGB_ERR_BOUNDS.  compute-sanitizer is closed on this machine; this
checks reads as well as writes on the kernels' real launch shapes: the
single operators, both Poisson forms, solver steps, rollouts (tiled and
row-streaming stencils, column bands with halo groups at N=4096, graph
chunks, the fused row kernel), checkpointed gradients with the tiled and the
row-streaming adjoint, an ensemble (graph chunks and the persistent launch), a
gradient batch and an optimiser loop.
The checker itself is exercised by registering a buffer shorter than the
kernel uses: the access beyond the registered end is reported (and skipped;
the buffer itself is long enough, so nothing touches invalid memory)."""
import ctypes
import math
import os

import numpy as np
import pytest
import torch

from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0

pytestmark = pytest.mark.gpu

L2PI = 2 * math.pi
ERR_BOUNDS = 7


@pytest.fixture(scope="module")
def chk(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _build, _native
    path = _build.build_checked()
    # linked -Bsymbolic: its calls stay inside it though libnsgb.so is loaded too
    C = ctypes.CDLL(path, mode=os.RTLD_LOCAL)
    for name, (args, res) in _native.SIGNATURES.items():
        fn = getattr(C, name)
        fn.argtypes = args
        fn.restype = res
    assert C.nsgb_bounds_checking() == 1 and cuda_lib.nsgb_bounds_checking() == 0
    return C, _native


class Ctx:
    """Registers device tensors with the checked library; plans are the
    checked library's own."""

    def __init__(self, C, nat):
        self.C, self.nat = C, nat
        self.keep = []
        self.plans = {}
        self.st = torch.cuda.current_stream().cuda_stream
        assert C.nsgb_bounds_clear() == 0

    def t(self, shape, dtype=torch.float32, fill=None):
        x = torch.empty(shape, dtype=dtype, device="cuda") if fill is None else fill.clone()
        self.reg(x)
        return x

    def reg(self, x, short=0):
        self.keep.append(x)
        assert self.C.nsgb_bounds_register(x.data_ptr(), x.numel() * x.element_size() - short) == 0

    def ws(self, nbytes):
        return self.t((max(int(nbytes), 16),), torch.uint8)

    def plan(self, N):
        if N not in self.plans:
            h = ctypes.c_void_p()
            assert self.C.nsgb_plan_create(N, L2PI, ctypes.byref(h)) == 0
            self.plans[N] = h
        return self.plans[N]

    def ok(self, rc):
        assert rc == 0, (rc, self.C.nsgb_last_error())

    def close(self):
        for h in self.plans.values():
            self.C.nsgb_plan_destroy(h)
        assert self.C.nsgb_bounds_clear() == 0


@pytest.fixture
def ctx(chk):
    c = Ctx(*chk)
    yield c
    c.close()


def _fields(ctx, N, seed=2):
    u0 = ctx.t(None, fill=torch.from_numpy(spectral_u0(N, min(8, N // 4), seed)).cuda())
    th = ctx.t(None, fill=torch.tensor([0.9, 0.4, 2e-3], dtype=torch.float32, device="cuda"))
    return u0, th


def _phys(ctx, scheme, dt, nu=2e-3):
    return ctx.nat.make_phys(L2PI, nu, dt, scheme)


@pytest.mark.parametrize("N", [64, 1024])
def test_operators_and_poisson(ctx, N):
    C, st, h = ctx.C, ctx.st, ctx.plan(N)
    u0, th = _fields(ctx, N)
    f = ctx.t((N, N), fill=u0[0].contiguous())
    gx, gy, lap, div = (ctx.t((N, N)) for _ in range(4))
    ctx.ok(C.nsgb_grad(h, f.data_ptr(), gx.data_ptr(), gy.data_ptr(), st))
    ctx.ok(C.nsgb_laplacian(h, f.data_ptr(), lap.data_ptr(), st))
    ctx.ok(C.nsgb_divergence(h, u0.data_ptr(), div.data_ptr(), st))
    for sid in (0, 1):
        out = ctx.t((N, N))
        ctx.ok(C.nsgb_advect(h, sid, f.data_ptr(), u0[0].data_ptr(), u0[1].data_ptr(), out.data_ptr(), st))
    force = ctx.t((2, N, N))
    ph = _phys(ctx, "central", 1e-3)
    ctx.ok(C.nsgb_forcing(h, ctypes.byref(ph), th.data_ptr(), 3, ctypes.c_float(0.3), force.data_ptr(), st))
    ws = ctx.ws(C.nsgb_poisson_workspace_bytes(h))
    p = ctx.t((N, N))
    ctx.ok(C.nsgb_poisson(h, div.data_ptr(), p.data_ptr(), ws.data_ptr(), ws.numel(), st))
    pn = ctx.t((N, N))
    ctx.ok(C.nsgb_poisson_noalloc(N, L2PI, div.data_ptr(), pn.data_ptr(), st))


@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_steps(ctx, scheme):
    C, st, N = ctx.C, ctx.st, 256
    h = ctx.plan(N)
    u0, th = _fields(ctx, N)
    ph = _phys(ctx, scheme, 1e-3)
    ws = ctx.ws(C.nsgb_step_workspace_bytes(h))
    out = ctx.t((2, N, N))
    ctx.ok(C.nsgb_step(h, ctypes.byref(ph), u0.data_ptr(), th.data_ptr(), 3, ctypes.c_float(0.01), out.data_ptr(),
                       ws.data_ptr(), ws.numel(), st))
    force = ctx.t((2, N, N))
    force.zero_()
    ctx.ok(C.nsgb_projector_step(h, ctypes.byref(ph), u0.data_ptr(), force.data_ptr(), out.data_ptr(),
                                 ws.data_ptr(), ws.numel(), st))


@pytest.mark.parametrize("N,tiles,fused,steps", [
    (64, (32, 8), 0, 40),            # tiled stencil, graph chunks
    (1024, (256, 24), 0, 5),         # row bands with halo groups
    (1024, (1024, 14), 14, 40),      # fused row kernel, graph chunks
    (4096, (2048, 54), 0, 3),        # the headline band shape
    (4096, (2048, 54), 54, 3),       # fused, two-CTA clusters
])
def test_rollout(ctx, N, tiles, fused, steps):
    C, st = ctx.C, ctx.st
    h = ctx.plan(N)
    ctx.ok(C.nsgb_plan_set_fft_radix(h, 16, 16))
    ctx.ok(C.nsgb_plan_set_tiles(h, tiles[0], tiles[1], 0, 0))
    ctx.ok(C.nsgb_plan_set_fused(h, fused))
    u0, th = _fields(ctx, N)
    ph = _phys(ctx, "upwind", 0.4 / N)
    ws = ctx.ws(C.nsgb_rollout_workspace_bytes(h, steps))
    uf, J = ctx.t((2, N, N)), ctx.t(())
    ctx.ok(C.nsgb_rollout(h, ctypes.byref(ph), u0.data_ptr(), th.data_ptr(), 3, steps, uf.data_ptr(), J.data_ptr(),
                          ws.data_ptr(), ws.numel(), 1, st))
    assert torch.isfinite(uf).all() and torch.isfinite(J)


@pytest.mark.parametrize("N,adj", [(64, (32, 8)), (1024, (1024, 8))])
def test_gradient(ctx, N, adj):
    C, st = ctx.C, ctx.st
    h = ctx.plan(N)
    ctx.ok(C.nsgb_plan_set_adjoint_tiles(h, adj[0], adj[1]))
    u0, th = _fields(ctx, N)
    ph = _phys(ctx, "upwind", 0.4 / N)
    steps, every = 9, 4
    ws = ctx.ws(C.nsgb_rollout_grad_workspace_bytes(h, steps, every))
    J, uf, g, du0 = ctx.t(()), ctx.t((2, N, N)), ctx.t((3,)), ctx.t((2, N, N))
    phases = ctx.nat.GRAD_FORWARD | ctx.nat.GRAD_BACKWARD
    ctx.ok(C.nsgb_rollout_grad(h, ctypes.byref(ph), u0.data_ptr(), th.data_ptr(), 3, steps, every, phases,
                               J.data_ptr(), uf.data_ptr(), g.data_ptr(), du0.data_ptr(), ws.data_ptr(), ws.numel(),
                               st))
    assert torch.isfinite(g).all()


def test_ensemble_and_gradient_batch(ctx):
    C, st, nat = ctx.C, ctx.st, ctx.nat
    sizes = [64, 128, 64, 256]
    arr = (nat.Member * len(sizes))()
    for k, N in enumerate(sizes):
        u0, th = _fields(ctx, N, seed=k)
        arr[k].plan = ctx.plan(N).value
        arr[k].phys = _phys(ctx, "central", 1e-3)
        arr[k].u0, arr[k].theta, arr[k].theta_len = u0.data_ptr(), th.data_ptr(), 3
        arr[k].u_final, arr[k].J = ctx.t((2, N, N)).data_ptr(), ctx.t(()).data_ptr()
        arr[k].state, arr[k].total_steps, arr[k].done_steps = None, 20, 0
    ws = ctx.ws(C.nsgb_ensemble_workspace_bytes(arr, len(sizes)))
    ctx.ok(C.nsgb_ensemble_rollout(arr, len(sizes), 8, ws.data_ptr(), ws.numel(), st))
    pws = ctx.ws(C.nsgb_ensemble_persistent_workspace_bytes(arr, len(sizes)))
    ctx.ok(C.nsgb_ensemble_persistent(arr, len(sizes), pws.data_ptr(), pws.numel(), st))

    cases = [(64, 9, 4, "upwind"), (128, 5, 2, "central"), (64, 3, 1, "central")]
    g_arr = (nat.GradMember * len(cases))()
    for k, (N, steps, every, scheme) in enumerate(cases):
        u0, th = _fields(ctx, N, seed=k)
        h = ctx.plan(N)
        m = g_arr[k]
        m.plan, m.phys = h.value, _phys(ctx, scheme, 0.4 / N)
        m.u0, m.theta, m.theta_len, m.steps, m.every = u0.data_ptr(), th.data_ptr(), 3, steps, every
        m.J, m.u_final, m.dJdtheta, m.dJdu0 = ctx.t(()).data_ptr(), None, ctx.t((3,)).data_ptr(), None
        m.state = ctx.ws(C.nsgb_rollout_grad_workspace_bytes(h, steps, every)).data_ptr()
        m.done_ops = 0
    ops = max(C.nsgb_grad_ops(s, e) for _, s, e, _ in cases)
    gws = ctx.ws(C.nsgb_grad_batch_workspace_bytes(len(cases), ops))
    ctx.ok(C.nsgb_grad_batch_advance(g_arr, len(cases), ops, gws.data_ptr(), gws.numel(), st))


def test_optimizer_loop(ctx):
    C, st, nat = ctx.C, ctx.st, ctx.nat
    N, steps, every, iters = 64, 6, 3, 3
    h = ctx.plan(N)
    u0, th = _fields(ctx, N)
    ph = _phys(ctx, "central", 1e-3)
    opt = nat.Optimizer(1, 0.05, 0.9, 0.999, 1e-8, 0.0, 0.9)  # adam
    ws = ctx.ws(C.nsgb_optimize_workspace_bytes(h, steps, every, 2))
    obj, par = ctx.t((iters + 1,)), ctx.t(((iters + 1) * 2,))
    ctx.ok(C.nsgb_optimize(h, ctypes.byref(ph), None, th.data_ptr(), 2, steps, every, ctypes.byref(opt), iters,
                           obj.data_ptr(), par.data_ptr(), ws.data_ptr(), ws.numel(), st))
    assert torch.isfinite(obj).all()


def test_checker_reports_access_beyond_registered_end(ctx):
    """A buffer registered 16 bytes shorter than the kernel writes (output) or
    reads (input): the library returns NSGB_ERR_BOUNDS naming an address in
    the unregistered tail; correct registrations pass again afterwards."""
    C, st, N = ctx.C, ctx.st, 64
    h = ctx.plan(N)
    f = ctx.t(None, fill=torch.randn(N, N, device="cuda"))
    out = torch.empty(N, N, device="cuda")
    ctx.reg(out, short=16)
    rc = C.nsgb_laplacian(h, f.data_ptr(), out.data_ptr(), st)
    msg = C.nsgb_last_error().decode()
    assert rc == ERR_BOUNDS and "out-of-range" in msg, msg
    end = out.data_ptr() + out.numel() * 4
    addr = int(msg.split("address ")[1].split()[0], 16)
    assert end - 16 <= addr < end, (hex(addr), hex(end))
    assert "4 access(es)" in msg  # the last four cells, one float store each
    assert C.nsgb_bounds_unregister(out.data_ptr()) == 0
    ctx.reg(out)
    ctx.ok(C.nsgb_laplacian(h, f.data_ptr(), out.data_ptr(), st))
    # an input read beyond its registered end
    g = torch.randn(N, N, device="cuda")
    ctx.reg(g, short=16)
    rc = C.nsgb_laplacian(h, g.data_ptr(), out.data_ptr(), st)
    assert rc == ERR_BOUNDS and "out-of-range" in C.nsgb_last_error().decode()
    # the normal build's calls are no-ops and say so
    from ns_solver_jax_differential_distributed_gb300 import _native
    assert _native.lib().nsgb_bounds_register(g.data_ptr(), 16) == 0
    assert np.isfinite(out.cpu().numpy()).all()
