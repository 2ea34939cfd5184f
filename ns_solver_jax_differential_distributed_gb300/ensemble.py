"""Ensembles of independent solves of uneven grid size, advanced together.

``Ensemble.run()`` calls ``nsgb_ensemble_rollout``: members that share N and
scheme form a group, every stage of a solver step is one batched launch per
group, and chunks of steps replay as one CUDA graph in which the groups are
parallel branches.  Each member's result equals its own plain
``SingleCoreNSSolver.rollout`` (the per-member arithmetic and reduction order
do not depend on the ensemble), which the tests check bit for bit.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _native, autotune


Member = _native.Member


def _bind():
    return _native.lib()


@dataclass
class SolveSpec:
    """One member: grid size, parameters and initial state."""
    N: int
    u0: np.ndarray
    theta: np.ndarray
    nu: float
    dt: float
    scheme: str = "central"
    L: float = 2 * math.pi
    mu0: float = 0.5
    sigma0: float = 0.1
    C: float = 1.0


class Ensemble:
    """Device-resident ensemble; ``run()`` advances all members by ``steps``."""

    def __init__(self, specs, steps: int, device=None, chunk: int = 16, tune: bool = False):
        self.device = torch.device(device or "cuda")
        self.steps = int(steps)
        self.chunk = int(chunk)
        self.specs = list(specs)
        if tune:
            for N, scheme, L in sorted({(s.N, s.scheme, s.L) for s in self.specs}):
                autotune.tune(N, L, scheme, self.device)
        else:
            for N, scheme, L in sorted({(s.N, s.scheme, s.L) for s in self.specs}):
                autotune.apply_cached(N, L, scheme, self.device)
        self.u0 = [torch.from_numpy(np.ascontiguousarray(s.u0, dtype=np.float32)).to(self.device)
                   for s in self.specs]
        for k, (s, u) in enumerate(zip(self.specs, self.u0)):
            # the kernels read each member's field through a bare pointer
            if tuple(u.shape) != (2, s.N, s.N):
                raise ValueError(f"member {k}: u0 must have shape (2, {s.N}, {s.N}), got {tuple(u.shape)}")
        self.theta = [torch.from_numpy(np.asarray(s.theta, dtype=np.float32)).to(self.device)
                      for s in self.specs]
        self.u_final = [torch.empty_like(u) for u in self.u0]
        self.J = torch.empty(len(self.specs), dtype=torch.float32, device=self.device)
        arr = (Member * len(self.specs))()
        for k, s in enumerate(self.specs):
            plan = _native.get_plan(s.N, s.L, self.device)
            arr[k].plan = plan.handle.value
            arr[k].phys = _native.make_phys(s.L, s.nu, s.dt, s.scheme, s.mu0, s.sigma0, s.C)
            arr[k].u0 = self.u0[k].data_ptr()
            arr[k].theta = self.theta[k].data_ptr()
            arr[k].theta_len = self.theta[k].numel()
            arr[k].u_final = self.u_final[k].data_ptr()
            arr[k].J = self.J.data_ptr() + 4 * k
            arr[k].state = None
            arr[k].total_steps = self.steps
            arr[k].done_steps = 0
        self._members = arr
        self.workspace = torch.empty(0, dtype=torch.uint8, device=self.device)
        self._ensure_workspace()
        if tune:
            self.tune_batched()

    def _ensure_workspace(self) -> None:
        """Size the workspace for the plans' current launch shapes."""
        nbytes = _bind().nsgb_ensemble_workspace_bytes(self._members, len(self.specs))
        if nbytes == 0:
            raise ValueError("invalid ensemble")
        if self.workspace.numel() < nbytes:
            self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=self.device)

    def _time_run(self) -> float:
        self.run()
        torch.cuda.synchronize(self.device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        self.run()
        e1.record()
        torch.cuda.synchronize(self.device)
        return e0.elapsed_time(e1)

    def tune_batched(self) -> None:
        """Choose each grid size's stencil shape for batched launches by timing
        the whole ensemble: the single-solve tuner favours short row bands
        (one solve must fill the GPU), while a batch gets its parallelism from
        its members and prefers taller bands, whose halo overhead is smaller.
        Then, per size, the FFT passes' CTA shapes (rows per CTA) the same
        way; the radix stays as tuned for single solves, so fields keep the
        bits of single solves.  Largest groups first.
        The shapes are set on the plans the process shares per grid size, so
        later solves of those sizes use them too (fields keep their bits; J
        can change by rounding, its partials following the stencil's blocks);
        ``autotune.apply_cached`` restores the single-solve shapes."""
        cells = {}
        for s in self.specs:
            cells[(s.N, s.L)] = cells.get((s.N, s.L), 0) + s.N * s.N
        for (N, L) in sorted(cells, key=cells.get, reverse=True):
            plan = _native.get_plan(N, L, self.device)
            base = plan.tiles()
            cands = [tuple(base[:2])]
            if N >= 64:
                cands += [(64, 16), (128, 8)] if N >= 128 else [(64, 16)]
            if N >= 128:
                cands += [(max(256, min(512, N)), h) for h in (16, 32) if h <= N]
            best, best_ms = tuple(base[:2]), None
            for (tw, th) in dict.fromkeys(cands):
                try:
                    plan.set_tiles(tw, th, base[2], base[3])
                except _native.NativeError:
                    continue
                self._ensure_workspace()
                ms = min(self._time_run() for _ in range(2))  # the better of two: less timing noise
                if best_ms is None or ms < best_ms:
                    best, best_ms = (tw, th), ms
            # the FFT passes' CTA shapes for the batch: rows of a row-FFT CTA,
            # then spectrum rows of a column CTA.  The radix stays and rows
            # are paired the same way in any shape, so every transform keeps
            # its bits.
            shape = [base[2], base[3]]
            for axis, choices in ((0, autotune.ROW_CHOICES), (1, autotune.COL_CHOICES)):
                keep, keep_ms = shape[axis], None
                for v in choices:
                    trial = list(shape)
                    trial[axis] = v
                    try:
                        plan.set_tiles(best[0], best[1], trial[0], trial[1])
                    except _native.NativeError:
                        continue
                    self._ensure_workspace()
                    ms = min(self._time_run() for _ in range(2))
                    if keep_ms is None or ms < keep_ms:
                        keep, keep_ms = v, ms
                shape[axis] = keep
            plan.set_tiles(best[0], best[1], shape[0], shape[1])
            self._ensure_workspace()

    @property
    def cell_steps(self) -> int:
        return sum(s.N * s.N for s in self.specs) * self.steps

    def run(self):
        """Advance every member; returns (J[count], [u_final...])."""
        self._ensure_workspace()
        L = _bind()
        _native.check("nsgb_ensemble_rollout", L.nsgb_ensemble_rollout(
            self._members, len(self.specs), self.chunk, self.workspace.data_ptr(),
            self.workspace.numel(), _native.stream_of(self.device)))
        return self.J, self.u_final

    def run_persistent(self):
        """The same ensemble in ONE persistent cooperative launch
        (``nsgb_ensemble_persistent``): fields equal ``run()``'s with radix-16
        transforms bit for bit; J to rounding (its partials follow 64 x 16
        tiles).  N a power of two in [64, 4096]."""
        L = _bind()
        need = L.nsgb_ensemble_persistent_workspace_bytes(self._members, len(self.specs))
        if need == 0:
            raise _native.NativeError("nsgb_ensemble_persistent_workspace_bytes", 1,
                                      "members outside the persistent launch's sizes (64..4096)")
        if getattr(self, "_pws", None) is None or self._pws.numel() < need:
            self._pws = torch.empty(need, dtype=torch.uint8, device=self.device)
        _native.check("nsgb_ensemble_persistent", L.nsgb_ensemble_persistent(
            self._members, len(self.specs), self._pws.data_ptr(), self._pws.numel(), _native.stream_of(self.device)))
        return self.J, self.u_final

    def run_advance(self, steps_per_call: int):
        """The same ensemble through nsgb_ensemble_advance in slices of
        ``steps_per_call`` steps (the continuous-batching entry point)."""
        self._ensure_workspace()
        L = _bind()
        done = 0
        while True:
            for k in range(len(self.specs)):
                self._members[k].done_steps = done
            _native.check("nsgb_ensemble_advance", L.nsgb_ensemble_advance(
                self._members, len(self.specs), int(steps_per_call), self.workspace.data_ptr(),
                self.workspace.numel(), _native.stream_of(self.device)))
            done = min(self.steps, done + int(steps_per_call))
            if done >= self.steps:
                break
        return self.J, self.u_final

    def run_sequential(self):
        """The same members as one plain rollout each (the comparison path)."""
        Js, us = [], []
        for s, u0, th in zip(self.specs, self.u0, self.theta):
            J, u = _native.op_rollout(u0, th, self.steps, float(s.L), float(s.nu), float(s.dt),
                                      _native.SCHEME_IDS[s.scheme], float(s.mu0), float(s.sigma0),
                                      float(s.C), True)
            Js.append(J)
            us.append(u)
        return torch.stack(Js), us


def from_workload(members, scheme: str = None):
    """SolveSpecs from ``workloads.ensemble()`` members (their own scheme
    unless `scheme` is given)."""
    return [SolveSpec(N=m.N, u0=m.u0(), theta=m.theta, nu=m.nu, dt=m.dt, scheme=scheme or m.scheme, L=m.L)
            for m in members]


class GradientBatch:
    """Gradient solves (forward with checkpoints + discrete adjoint, the
    work of ``SingleCoreNSSolver.jit_gradient`` for a given u0) advanced
    together by ``nsgb_grad_batch_advance``.  Solves may join at any call
    (continuous batching); each solve's J and dJ/dtheta equal its own
    ``nsgb_rollout_grad`` bit for bit.

    ``add`` returns a solve id; ``advance(ops)`` moves every unfinished solve
    by up to ``ops`` operations of its schedule (a forward, recomputed or
    adjoint step each) and returns the ids that completed; ``result(id)``
    gives (J, dJ/dtheta) as device tensors."""

    def __init__(self, device=None):
        self.device = torch.device(device or "cuda")
        self._solves = {}
        self._next = 0
        self._ws = None

    def add(self, u0, theta, steps: int, every: int, L: float, nu: float, dt: float, scheme,
            mu0: float = 0.5, sigma0: float = 0.1, C: float = 1.0, want_du0: bool = False,
            want_u_final: bool = False) -> int:
        u0 = _native._cuda_f32(torch.as_tensor(u0, dtype=torch.float32).to(self.device), "u0")
        theta = _native._cuda_f32(torch.as_tensor(theta, dtype=torch.float32).to(self.device), "theta")
        N = _native._square(u0, "u0", 2)
        if theta.numel() not in (2, 3):
            raise ValueError(f"theta must have 2 or 3 entries, got {theta.numel()}")
        steps, every = int(steps), int(every)
        if steps < 1 or every < 1:
            raise ValueError(f"steps and every must be >= 1, got {steps} and {every}")
        phys = _native.make_phys(L, nu, dt, scheme, mu0, sigma0, C)
        plan = _native.get_plan(N, L, self.device)
        lib = _bind()
        state = torch.empty(lib.nsgb_rollout_grad_workspace_bytes(plan.handle, steps, every),
                            dtype=torch.uint8, device=self.device)
        m = _native.GradMember()
        m.plan = plan.handle.value
        m.phys = phys
        rec = {
            "u0": u0, "theta": theta, "plan": plan, "state": state,
            "J": torch.empty((), dtype=torch.float32, device=self.device),
            "g": torch.empty(theta.numel(), dtype=torch.float32, device=self.device),
            "du0": torch.empty_like(u0) if want_du0 else None,
            "u_final": torch.empty_like(u0) if want_u_final else None,
            "total": int(lib.nsgb_grad_ops(steps, every)), "member": m,
        }
        m.u0 = u0.data_ptr()
        m.theta = theta.data_ptr()
        m.theta_len = theta.numel()
        m.steps, m.every = steps, every
        m.J = rec["J"].data_ptr()
        m.u_final = rec["u_final"].data_ptr() if want_u_final else None
        m.dJdtheta = rec["g"].data_ptr()
        m.dJdu0 = rec["du0"].data_ptr() if want_du0 else None
        m.state = state.data_ptr()
        m.done_ops = 0
        sid = self._next
        self._next += 1
        self._solves[sid] = rec
        return sid

    def pending(self):
        return [k for k, r in self._solves.items() if r["member"].done_ops < r["total"]]

    def advance(self, ops: int):
        ids = self.pending()
        if not ids or ops <= 0:
            return []
        lib = _bind()
        arr = (_native.GradMember * len(ids))(*[self._solves[k]["member"] for k in ids])
        need = lib.nsgb_grad_batch_workspace_bytes(len(ids), int(ops))
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        _native.check("nsgb_grad_batch_advance", lib.nsgb_grad_batch_advance(
            arr, len(ids), int(ops), self._ws.data_ptr(), self._ws.numel(), _native.stream_of(self.device)))
        done = []
        for k in ids:
            r = self._solves[k]
            r["member"].done_ops = min(r["total"], r["member"].done_ops + int(ops))
            if r["member"].done_ops == r["total"]:
                done.append(k)
        return done

    def run(self, ops_per_call: int = 64):
        while self.pending():
            self.advance(ops_per_call)

    def _finished(self, sid: int) -> dict:
        r = self._solves[sid]
        if r["member"].done_ops < r["total"]:
            raise RuntimeError(f"gradient solve {sid} has done {r['member'].done_ops} of its "
                               f"{r['total']} operations")
        return r

    def result(self, sid: int):
        r = self._finished(sid)
        return r["J"], r["g"]

    def du0(self, sid: int):
        return self._finished(sid)["du0"]

    def u_final(self, sid: int):
        """The final state (written when the forward phase ends)."""
        return self._finished(sid)["u_final"]

    def release(self, sid: int):
        """Frees a finished (or abandoned) solve's device state."""
        self._solves.pop(sid, None)
