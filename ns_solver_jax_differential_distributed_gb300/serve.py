"""Serving loop: continuous batching of forward and gradient solves.

Requests (N, steps, theta, u0, forward-only or forward+adjoint) arrive over
time.  A scheduler thread owns the GPU:

* admission -- a request is admitted (FIFO) when its device memory (state,
  u0, outputs) fits the HBM budget and the active forward work stays under a
  cap; it then keeps its fields resident on the device until it completes;
* forward requests are continuously batched: each tick advances every
  active forward request by up to ``slice_steps`` steps in one
  ``nsgb_ensemble_advance`` call (one batched launch per stage per group of
  equal N), so requests that arrive while others run join at the next tick;
* gradient requests (forward with checkpoints + discrete adjoint) are
  continuously batched the same way on a second CUDA stream: each tick moves
  every active gradient request by up to ``grad_slice_ops`` operations of its
  schedule in one ``nsgb_grad_batch_advance`` call (one batched launch per
  kernel per group of equal N), overlapping the forward tick on the device;
  ``grad_mode="workers"`` instead runs each one as ``nsgb_rollout_grad`` on
  worker threads with their own streams;
* completion is detected with CUDA events; memory returns to the budget.

Failures are isolated per request: every request ends with a ``status`` --
"ok", "nonfinite" (its objective or gradient is not finite, e.g. a NaN in its
initial state; NSGB_ERR_NONFINITE of the C ABI), "failed" (its allocation or
its solve raised; ``error`` says why) or "cancelled" (``Server.cancel``) --
and the others carry on with the same results as when served alone.

``Server.stop`` ends a run gracefully: the active forward and batched
gradient requests are suspended to host memory (status "suspended", their
device state, J and progress in ``Request.resume``), requests not yet
admitted come back with status "queued", and a later ``run`` given them
resumes each where it stopped, with the bits of an uninterrupted solve.  A
run that reaches its drain limit ends the same way.

Latency is measured from arrival to the moment the result (J, and dJ/dtheta
for gradient requests) is on the host; for a resumed request, from the start
of the run that resumed it.  Results do not depend on what else
is in flight: a request's arithmetic is that of a plain solve, which the
tests check bit for bit.
"""
from __future__ import annotations

import collections
import math
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native
from .workloads import spectral_u0, theta_draw

TWO_PI = 2.0 * math.pi


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the trace
    N: int
    steps: int
    kind: str               # "forward" or "grad"
    seed: int
    nu: float = 1e-3
    dt: float = 1e-3
    scheme: str = "central"
    L: float = TWO_PI
    theta: np.ndarray = None
    # results
    J: float = None
    grad: np.ndarray = None
    u_final: torch.Tensor = field(default=None, repr=False)
    t_admit: float = None
    t_done: float = None
    status: str = None      # "ok", "nonfinite", "failed", "cancelled", "suspended", "queued"
    error: str = None
    u0: torch.Tensor = field(default=None, repr=False)  # explicit initial state (else seeded)
    # a suspended request's host checkpoint: its device state, J, progress
    # (steps or gradient operations done) and the launch shapes it ran with
    resume: dict = field(default=None, repr=False)

    @property
    def cells(self) -> int:
        return self.N * self.N * self.steps

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


# Time step of a request without an explicit one: the reference's stable step
# (SimConfig.dt, NS_solver.py:75-79), min(cfl dx / v_max, dx^2 / (4 nu)) rounded
# through float32, with its cfl of 0.4 and v_max = 4, a bound on the speed of
# the seeded initial states (rms 1, maximum about 3).
STABLE_CFL, STABLE_VMAX = 0.4, 4.0


def stable_dt(N: int, L: float, nu: float) -> float:
    dx = L / N
    return float(np.float32(min(STABLE_CFL * dx / STABLE_VMAX, dx * dx / (4.0 * nu))))


def make_trace(rate: float = 200.0, duration: float = 60.0, seed: int = 7,
               sizes=(128, 256, 512, 1024, 2048), steps_range=(100, 2000), p_grad: float = 0.3,
               dt: float = None, nu_default: float = 1e-3, scheme: str = "upwind"):
    """Poisson arrivals; N uniform over `sizes` (log-uniform over the
    power-of-two set), steps uniform in `steps_range`, gradient with
    probability `p_grad`; theta (and with it nu) seeded per request; dt the
    stable step of each request's N and nu unless given.  Upwind advection by
    default: with central differences and forward Euler, runs of up to 2000
    steps at these viscosities grow grid-scale modes until they overflow
    (N = 512 already at the stable step), which upwind differencing damps."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        rid = len(out)
        N = int(rng.choice(np.asarray(sizes)))
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        kind = "grad" if rng.random() < p_grad else "forward"
        th = theta_draw(nu_default, seed=rid)
        nu = float(th[2])
        step = stable_dt(N, TWO_PI, nu) if dt is None else dt
        out.append(Request(rid, t, N, steps, kind, rid, nu=nu, dt=step, scheme=scheme, theta=th))
    return out


class _U0Cache:
    """Seeded initial states; requests share 16 seeds per N (the generator
    costs far more host time than a request's arrival interval at N=2048)."""

    def __init__(self, device, K=32, variants=16):
        self.device, self.K, self.variants = device, K, variants
        self._c = {}
        self._lock = threading.Lock()

    def get(self, N: int, seed: int) -> torch.Tensor:
        key = (N, seed % self.variants)
        with self._lock:
            if key not in self._c:
                t = torch.from_numpy(spectral_u0(N, min(self.K, N // 4), key[1])).to(self.device)
                torch.cuda.synchronize(self.device)  # shared by all streams afterwards
                self._c[key] = t
            return self._c[key]


GRAD_EVERY = 50  # checkpoint interval of served gradient requests


class Server:
    def __init__(self, device=None, hbm_budget: float = 150e9, slice_steps: int = 32,
                 max_active_cells: float = 96 * 2 ** 20, grad_workers: int = 8,
                 grad_mode: str = "batched", grad_slice_ops: int = 32,
                 max_active_grad_cells: float = 48 * 2 ** 20):
        if grad_mode not in ("batched", "workers"):
            raise ValueError(f"grad_mode must be 'batched' or 'workers', got {grad_mode!r}")
        dev = torch.device(device or "cuda")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        self.budget = float(hbm_budget)
        self.slice = int(slice_steps)
        self.max_active_cells = float(max_active_cells)
        self.grad_workers = int(grad_workers)
        self.grad_mode = grad_mode
        self.grad_slice = int(grad_slice_ops)
        self.max_active_grad_cells = float(max_active_grad_cells)
        self.u0 = _U0Cache(self.device)
        self.used = 0.0
        self.peak_used = 0.0
        self.stats = collections.Counter()
        self._lock = threading.Lock()
        self._cancel = set()
        self._stop = False

    def cancel(self, rid: int) -> None:
        """Cancel request `rid`: dropped if still queued or advancing in a
        batch (its memory returns to the budget at the next tick); a gradient
        already running on a worker thread (grad_mode="workers") completes and
        is then reported cancelled."""
        with self._lock:
            self._cancel.add(int(rid))

    def _cancelled(self, r: Request) -> bool:
        with self._lock:
            return r.rid in self._cancel

    def stop(self) -> None:
        """Ask the running ``run`` (any thread may call this) to stop at its
        next pass: it admits nothing more, suspends its active forward and
        batched gradient requests to host memory, lets gradients already on
        worker threads finish, and returns every request it was given, the
        unfinished ones with status "suspended" or "queued"."""
        with self._lock:
            self._stop = True

    def _stopping(self) -> bool:
        with self._lock:
            return self._stop

    # -- checkpoints of suspended requests
    @staticmethod
    def _shapes(plan) -> tuple:
        # the objective partials are laid out by the stencil's launch shape,
        # so a state resumes only under the shapes it was written with
        return (plan.tiles(), plan.fft_radix(), plan.adjoint_tiles(), plan.fused_rows())

    def _suspend(self, r: Request, plan, state: torch.Tensor, J: torch.Tensor, progress: int, stream) -> None:
        host = torch.empty(state.shape, dtype=torch.uint8, pin_memory=True)
        Jh = torch.empty((), dtype=torch.float32, pin_memory=True)
        with torch.cuda.stream(stream):
            host.copy_(state, non_blocking=True)
            Jh.copy_(J, non_blocking=True)
        r.resume = {"state": host, "J": Jh, "progress": int(progress), "shapes": self._shapes(plan)}
        r.status, r.t_done = "suspended", None

    def _restore(self, r: Request, plan, state: torch.Tensor, J: torch.Tensor, stream) -> int:
        """Copy a suspended request's checkpoint into its new device state;
        returns its progress."""
        res = r.resume
        if res["shapes"] != self._shapes(plan):
            raise RuntimeError(f"the launch shapes of N={r.N} changed since request {r.rid} was suspended "
                               f"({res['shapes']} -> {self._shapes(plan)})")
        if res["state"].numel() != state.numel():
            raise RuntimeError(f"request {r.rid}: checkpoint of {res['state'].numel()} bytes, "
                               f"state of {state.numel()}")
        with torch.cuda.stream(stream):
            state.copy_(res["state"], non_blocking=True)
            J.copy_(res["J"], non_blocking=True)
        return int(res["progress"])

    def _alloc(self, r: Request, shape, dtype) -> torch.Tensor:
        """Device allocation of a request's resident fields (a test may
        replace it to inject allocation failures)."""
        return torch.empty(shape, dtype=dtype, device=self.device)

    def _initial(self, r: Request) -> torch.Tensor:
        return r.u0 if r.u0 is not None else self.u0.get(r.N, r.seed)

    def _prepare(self, r: Request) -> None:
        """Checks of a request's own arguments on arrival, so that a bad
        request fails alone instead of stopping the batch it would join: its
        kind, scheme, dt, nu and L (the C ABI's rules), steps >= 1, an N the
        kernels support, theta of 2 or 3 entries (kept as float32; none means
        the reference's default [1, 0.5]) and an explicit u0 of shape
        (2, N, N) in float32 on the server's device (copied when it is not
        contiguous or not 16-byte aligned)."""
        if r.kind not in ("forward", "grad"):
            raise ValueError(f"kind must be 'forward' or 'grad', got {r.kind!r}")
        _native.make_phys(r.L, r.nu, r.dt, r.scheme)  # raises on an unknown scheme
        for name, v in (("dt", r.dt), ("L", r.L)):
            if not (math.isfinite(v) and v > 0):
                raise ValueError(f"{name} must be positive and finite, got {v}")
        if not math.isfinite(r.nu):
            raise ValueError(f"nu must be finite, got {r.nu}")
        if int(r.steps) < 1:
            raise ValueError(f"steps must be >= 1, got {r.steps}")
        th = np.asarray([1.0, 0.5] if r.theta is None else r.theta, dtype=np.float32).reshape(-1)
        if th.size not in (2, 3):
            raise ValueError(f"theta must have 2 or 3 entries, got {th.size}")
        r.theta = th
        _native.get_plan(r.N, r.L, self.device)  # raises on an unsupported N
        if r.u0 is not None:
            u0 = _native._cuda_f32(r.u0, "u0")
            if tuple(u0.shape) != (2, r.N, r.N) or u0.device != self.device:
                raise ValueError(f"u0 must be a (2, {r.N}, {r.N}) tensor on {self.device}, got "
                                 f"{tuple(u0.shape)} on {u0.device}")
            r.u0 = u0

    def _fail(self, r: Request, exc: BaseException, t0: float, completed: list) -> None:
        r.status, r.error = "failed", f"{type(exc).__name__}: {exc}"
        r.t_done = time.perf_counter() - t0
        completed.append(r)
        self.stats["failed"] += 1

    # -- memory accounting
    def _fwd_bytes(self, r: Request) -> int:
        plan = _native.get_plan(r.N, r.L, self.device)
        st = _native.lib().nsgb_rollout_workspace_bytes(plan.handle, r.steps)
        return int(st + 8 * r.N * r.N + 4096)  # state + u_final

    def _grad_bytes(self, r: Request) -> int:
        plan = _native.get_plan(r.N, r.L, self.device)
        return int(_native.lib().nsgb_rollout_grad_workspace_bytes(plan.handle, r.steps, GRAD_EVERY) + 4096)

    # -- gradient workers
    def _grad_worker(self, q: "queue.Queue", done_q: "queue.Queue"):
        torch.cuda.set_device(self.device)
        stream = torch.cuda.Stream(self.device)
        while True:
            item = q.get()
            if item is None:
                return
            r, nbytes = item
            try:
                with torch.cuda.stream(stream):
                    u0 = self._initial(r)
                    th = torch.from_numpy(r.theta).to(self.device, non_blocking=True)
                    J, g, _, _ = _native.rollout_grad_raw(u0, th, r.steps, GRAD_EVERY, r.L, r.nu, r.dt, r.scheme,
                                                          want_u_final=False, own_workspace=True)
                    Jh, gh = J.to("cpu", non_blocking=True), g.to("cpu", non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(stream)
                ev.synchronize()
                r.J, r.grad = float(Jh), gh.numpy().copy()
                done_q.put((r, nbytes, None))
            except Exception as exc:  # this request fails; the worker serves on
                done_q.put((r, nbytes, exc))

    def _admit_grad(self, r: Request, gstream) -> dict:
        """Device state of a batched gradient request, allocated on the
        gradient stream (raises if an allocation fails)."""
        L = _native.lib()
        with torch.cuda.stream(gstream):
            plan = _native.get_plan(r.N, r.L, self.device)
            st_bytes = L.nsgb_rollout_grad_workspace_bytes(plan.handle, r.steps, GRAD_EVERY)
            state = self._alloc(r, (st_bytes,), torch.uint8)
            th = torch.from_numpy(np.asarray(r.theta, dtype=np.float32)).to(self.device)
            J = self._alloc(r, (), torch.float32)
            g = self._alloc(r, (th.numel(),), torch.float32)
            u0 = self._initial(r)
        m = _native.GradMember()
        m.plan = plan.handle.value
        m.phys = _native.make_phys(r.L, r.nu, r.dt, r.scheme)
        m.u0 = u0.data_ptr()
        m.theta = th.data_ptr()
        m.theta_len = th.numel()
        m.steps, m.every = r.steps, GRAD_EVERY
        m.J, m.u_final, m.dJdtheta, m.dJdu0 = J.data_ptr(), None, g.data_ptr(), None
        m.state = state.data_ptr()
        m.done_ops = self._restore(r, plan, state, J, gstream) if r.resume is not None else 0
        return dict(r=r, m=m, state=state, th=th, J=J, g=g, u0=u0, plan=plan,
                    total=int(L.nsgb_grad_ops(r.steps, GRAD_EVERY)))

    def run(self, requests, realtime: bool = True, drain_limit: float = None, t0: float = None,
            suspend: bool = True):
        """Serve `requests` (sorted by arrival).  With realtime, arrivals
        follow the wall clock; otherwise all are available at once.  Stops
        when all are done, `drain_limit` seconds after the last arrival, or
        after ``stop()``; returns (requests, queue trace) with every request
        given, those left unfinished as "suspended" (a host checkpoint in
        ``resume``) or "queued".  Suspended requests passed again resume
        where they stopped (a gradient request served by worker threads
        starts over).  With ``suspend=False`` the active requests come back
        "queued", without host copies, and start over when passed again."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        pending = collections.deque()
        nxt = 0
        active = []          # forward requests: dict(r, state, done, out, J)
        grad_q, grad_done = queue.Queue(), queue.Queue()
        batched = self.grad_mode == "batched"
        workers = [] if batched else [
            threading.Thread(target=self._grad_worker, args=(grad_q, grad_done), daemon=True)
            for _ in range(self.grad_workers)]
        gstream = torch.cuda.Stream(self.device) if batched else None
        gactive = []         # batched gradient requests: dict(r, m, state, ...)
        gfinishing = []      # (event, entry, J on host, dJ/dtheta on host)
        gws = None
        gticks = collections.deque()
        for w in workers:
            w.start()
        grads_inflight = 0
        finishing = []       # (event, r, nbytes, J tensor)
        last_arrival = reqs[-1].arrival if reqs else 0.0
        t0 = time.perf_counter() if t0 is None else t0
        L = _native.lib()
        ws = None
        stream = torch.cuda.current_stream(self.device)
        completed = []
        queue_trace = []
        ticks = collections.deque()  # events of the ticks still on the GPU

        def collect():
            """Requests whose work has finished on the device."""
            nonlocal finishing, gfinishing, grads_inflight
            still = []
            for ev, a in finishing:
                if ev.query():
                    r = a["r"]
                    r.J = float(a["J_host"])
                    r.u_final = a["out"]
                    r.status = "ok" if math.isfinite(r.J) else "nonfinite"
                    r.t_done, r.resume = time.perf_counter() - t0, None
                    self.used -= a["nb"]
                    completed.append(r)
                else:
                    still.append((ev, a))
            finishing = still
            still = []
            for ev, a, Jh, gh in gfinishing:
                if ev.query():
                    r = a["r"]
                    r.J, r.grad = float(Jh), gh.numpy().copy()
                    if self._cancelled(r):
                        r.status = "cancelled"
                    else:
                        ok = math.isfinite(r.J) and bool(np.all(np.isfinite(r.grad)))
                        r.status = "ok" if ok else "nonfinite"
                    r.t_done, r.resume = time.perf_counter() - t0, None
                    self.used -= a["nb"]
                    grads_inflight -= 1
                    completed.append(r)
                else:
                    still.append((ev, a, Jh, gh))
            gfinishing = still
            while not grad_done.empty():
                r, nb, exc = grad_done.get()
                if exc is not None:
                    r.status, r.error = "failed", f"{type(exc).__name__}: {exc}"
                    self.stats["failed"] += 1
                elif self._cancelled(r):
                    r.status = "cancelled"
                else:
                    ok = math.isfinite(r.J) and bool(np.all(np.isfinite(r.grad)))
                    r.status = "ok" if ok else "nonfinite"
                r.t_done, r.resume = time.perf_counter() - t0, None
                self.used -= nb
                grads_inflight -= 1
                completed.append(r)

        while True:
            if self._stopping():
                break
            now = time.perf_counter() - t0
            while nxt < len(reqs) and (not realtime or reqs[nxt].arrival <= now):
                r = reqs[nxt]
                nxt += 1
                try:
                    self._prepare(r)
                except Exception as exc:  # this request fails; nothing was charged
                    self._fail(r, exc, t0, completed)
                    continue
                pending.append(r)
            # admission (FIFO): memory budget, and a cap on active forward work
            act_cells = sum(a["r"].N ** 2 for a in active)
            grad_cells = sum(a["r"].N ** 2 for a in gactive)
            while pending and self._cancelled(pending[0]):
                r = pending.popleft()
                r.status, r.t_done = "cancelled", time.perf_counter() - t0
                completed.append(r)
            while pending:
                r = pending[0]
                if self._cancelled(r):
                    break  # dropped at the top of the next pass
                nb = self._grad_bytes(r) if r.kind == "grad" else self._fwd_bytes(r)
                if self.used + nb > self.budget:
                    break
                if r.kind == "forward" and act_cells + r.N ** 2 > self.max_active_cells and active:
                    break
                if r.kind == "grad" and not batched and grads_inflight >= 2 * self.grad_workers:
                    break
                if (r.kind == "grad" and batched and gactive
                        and grad_cells + r.N ** 2 > self.max_active_grad_cells):
                    break
                pending.popleft()
                r.t_admit = time.perf_counter() - t0
                if r.kind == "grad" and batched:
                    try:
                        entry = self._admit_grad(r, gstream)
                    except Exception as exc:  # this request fails; nothing was charged
                        self._fail(r, exc, t0, completed)
                        continue
                    entry["nb"] = nb
                    self.used += nb
                    grads_inflight += 1
                    gactive.append(entry)
                    grad_cells += r.N ** 2
                elif r.kind == "grad":
                    self.used += nb
                    grads_inflight += 1
                    grad_q.put((r, nb))
                else:
                    try:
                        plan = _native.get_plan(r.N, r.L, self.device)
                        st_bytes = L.nsgb_rollout_workspace_bytes(plan.handle, r.steps)
                        state = self._alloc(r, (st_bytes,), torch.uint8)
                        out = self._alloc(r, (2, r.N, r.N), torch.float32)
                        Jt = self._alloc(r, (), torch.float32)
                        th = torch.from_numpy(r.theta).to(self.device)
                        done0 = self._restore(r, plan, state, Jt, stream) if r.resume is not None else 0
                    except Exception as exc:  # this request fails; nothing was charged
                        self._fail(r, exc, t0, completed)
                        continue
                    self.used += nb
                    active.append(dict(r=r, state=state, out=out, J=Jt, th=th, done=done0, nb=nb, plan=plan))
                    act_cells += r.N ** 2
                self.peak_used = max(self.peak_used, self.used)
            # cancelled requests leave before the next tick
            if gactive:
                keep = []
                for a in gactive:
                    if self._cancelled(a["r"]):
                        a["r"].status, a["r"].t_done = "cancelled", time.perf_counter() - t0
                        self.used -= a["nb"]
                        grads_inflight -= 1
                        completed.append(a["r"])
                    else:
                        keep.append(a)
                gactive = keep
            if active:
                keep = []
                for a in active:
                    if self._cancelled(a["r"]):
                        a["r"].status, a["r"].t_done = "cancelled", time.perf_counter() - t0
                        self.used -= a["nb"]
                        completed.append(a["r"])
                    else:
                        keep.append(a)
                active = keep
            # one tick of continuous batching over the active forward requests
            if active:
                arr = (_native.Member * len(active))()
                for k, a in enumerate(active):
                    r = a["r"]
                    arr[k].plan = a["plan"].handle.value
                    arr[k].phys = _native.make_phys(r.L, r.nu, r.dt, r.scheme)
                    arr[k].u0 = self._initial(r).data_ptr()
                    arr[k].theta = a["th"].data_ptr()
                    arr[k].theta_len = a["th"].numel()
                    arr[k].u_final = a["out"].data_ptr()
                    arr[k].J = a["J"].data_ptr()
                    arr[k].state = a["state"].data_ptr()
                    arr[k].total_steps = r.steps
                    arr[k].done_steps = a["done"]
                try:
                    need = L.nsgb_ensemble_workspace_bytes(arr, len(active))
                    if ws is None or ws.numel() < need:
                        ws = torch.empty(max(need, 1 << 20), dtype=torch.uint8, device=self.device)
                    _native.check("nsgb_ensemble_advance", L.nsgb_ensemble_advance(
                        arr, len(active), self.slice, ws.data_ptr(), ws.numel(), stream.cuda_stream))
                except Exception as exc:  # the tick's requests fail; the server serves on
                    for a in active:
                        self.used -= a["nb"]
                        self._fail(a["r"], exc, t0, completed)
                    active = []
                keep = []
                for a in active:
                    a["done"] = min(a["r"].steps, a["done"] + self.slice)
                    if a["done"] >= a["r"].steps:
                        a["J_host"] = a["J"].to("cpu", non_blocking=True)
                        ev = torch.cuda.Event()
                        ev.record(stream)
                        finishing.append((ev, a))
                    else:
                        keep.append(a)
                active = keep
                self.stats["ticks"] += 1
                # keep at most two ticks queued on the GPU, so admission and
                # the host's view of progress follow the device
                tev = torch.cuda.Event()
                tev.record(stream)
                ticks.append(tev)
                if len(ticks) > 2:
                    ticks.popleft().synchronize()
            # one tick of continuous batching over the active gradient requests
            if gactive:
                arr = (_native.GradMember * len(gactive))(*[a["m"] for a in gactive])
                need = L.nsgb_grad_batch_workspace_bytes(len(gactive), self.grad_slice)
                with torch.cuda.stream(gstream):
                    try:
                        if gws is None or gws.numel() < need:
                            gws = torch.empty(max(need, 1 << 20), dtype=torch.uint8, device=self.device)
                        _native.check("nsgb_grad_batch_advance", L.nsgb_grad_batch_advance(
                            arr, len(gactive), self.grad_slice, gws.data_ptr(), gws.numel(),
                            gstream.cuda_stream))
                    except Exception as exc:  # the tick's requests fail; the server serves on
                        for a in gactive:
                            self.used -= a["nb"]
                            grads_inflight -= 1
                            self._fail(a["r"], exc, t0, completed)
                        gactive = []
                    keep = []
                    for a in gactive:
                        a["m"].done_ops = min(a["total"], a["m"].done_ops + self.grad_slice)
                        if a["m"].done_ops >= a["total"]:
                            Jh = a["J"].to("cpu", non_blocking=True)
                            gh = a["g"].to("cpu", non_blocking=True)
                            ev = torch.cuda.Event()
                            ev.record(gstream)
                            gfinishing.append((ev, a, Jh, gh))
                        else:
                            keep.append(a)
                    gactive = keep
                    self.stats["grad_ticks"] += 1
                    tev = torch.cuda.Event()
                    tev.record(gstream)
                    gticks.append(tev)
                if len(gticks) > 2:
                    gticks.popleft().synchronize()
            collect()
            queue_trace.append((now, len(pending), len(active), grads_inflight))
            all_in = nxt >= len(reqs)
            if all_in and not pending and not active and not finishing and grads_inflight == 0:
                break
            if drain_limit is not None and now > last_arrival + drain_limit:
                break
            if not active and not finishing and not gactive and not gfinishing:
                time.sleep(0.0005)
        # The run ends: the active requests are suspended to host memory (their
        # copies follow their last tick on its stream), gradients waiting for a
        # worker thread go back to the queue, the running ones finish, and what
        # has finished on the device is collected.
        def park(a, progress, st):
            # a request whose checkpoint cannot be taken (no pinned host
            # memory) keeps its previous checkpoint if it has one, else comes
            # back queued and starts over
            if suspend:
                try:
                    self._suspend(a["r"], a["plan"], a["state"], a["J"], progress, st)
                    completed.append(a["r"])
                    return
                except Exception as exc:
                    a["r"].error = f"checkpoint failed: {type(exc).__name__}: {exc}"
            pending.append(a["r"])

        for a in active:
            park(a, a["done"], stream)
            self.used -= a["nb"]
        for a in gactive:
            park(a, a["m"].done_ops, gstream)
            self.used -= a["nb"]
            grads_inflight -= 1
        active, gactive = [], []
        while True:
            try:
                item = grad_q.get_nowait()
            except queue.Empty:
                break
            r, nb = item
            self.used -= nb
            grads_inflight -= 1
            pending.append(r)
        for _ in workers:
            grad_q.put(None)
        for w in workers:
            w.join()
        torch.cuda.synchronize(self.device)
        collect()
        for r in list(pending) + reqs[nxt:]:
            if self._cancelled(r):
                r.status, r.t_done = "cancelled", time.perf_counter() - t0
            else:
                r.status, r.t_done = ("suspended" if r.resume is not None else "queued"), None
            completed.append(r)
        with self._lock:
            self._stop = False
        return completed, queue_trace


def summarize(requests, completed, wall: float) -> dict:
    ok = [r for r in completed if r.status in (None, "ok")]
    lat = np.array([r.latency for r in ok if r.latency is not None])
    cells = sum(r.cells * (3.5 if r.kind == "grad" else 1.0) for r in ok)
    statuses = collections.Counter(r.status or "ok" for r in completed)
    return {
        "offered": len(requests), "completed": len(ok), "statuses": dict(statuses),
        "solves_per_s": len(ok) / wall if wall > 0 else 0.0,
        "p50_latency_s": float(np.percentile(lat, 50)) if lat.size else None,
        "p99_latency_s": float(np.percentile(lat, 99)) if lat.size else None,
        "forward_equiv_cell_steps_per_s": cells / wall if wall > 0 else 0.0,
        "wall_s": wall,
    }
