"""Binding of the C ABI (``include/nsgb.h``) and its registration as PyTorch ops.

The shared library is loaded with ctypes; torch supplies device memory
(tensors) and streams.  Every op here is registered for the CUDA device only,
so a call with CPU tensors raises instead of falling back to a CPU path, and a
missing ``libnsgb.so`` raises at first use.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

from . import _build

NSGB_OK = 0
SCHEME_IDS = {"central": 0, "upwind": 1}
GRAD_FORWARD = 1
GRAD_BACKWARD = 2

_lock = threading.RLock()
_lib = None


class Phys(ctypes.Structure):
    """``nsgb_phys`` (include/nsgb.h)."""
    _fields_ = [("L", ctypes.c_double), ("nu", ctypes.c_double), ("dt", ctypes.c_double),
                ("mu0", ctypes.c_double), ("sigma0", ctypes.c_double), ("C", ctypes.c_double),
                ("scheme", ctypes.c_int)]


class Member(ctypes.Structure):
    """``nsgb_member`` (include/nsgb.h): one solve of an ensemble."""
    _fields_ = [("plan", ctypes.c_void_p), ("phys", Phys), ("u0", ctypes.c_void_p),
                ("theta", ctypes.c_void_p), ("theta_len", ctypes.c_int), ("u_final", ctypes.c_void_p),
                ("J", ctypes.c_void_p), ("state", ctypes.c_void_p), ("total_steps", ctypes.c_int),
                ("done_steps", ctypes.c_int)]


class GradMember(ctypes.Structure):
    """``nsgb_grad_member`` (include/nsgb.h): one solve of a gradient batch."""
    _fields_ = [("plan", ctypes.c_void_p), ("phys", Phys), ("u0", ctypes.c_void_p),
                ("theta", ctypes.c_void_p), ("theta_len", ctypes.c_int), ("steps", ctypes.c_int),
                ("every", ctypes.c_int), ("J", ctypes.c_void_p), ("u_final", ctypes.c_void_p),
                ("dJdtheta", ctypes.c_void_p), ("dJdu0", ctypes.c_void_p), ("state", ctypes.c_void_p),
                ("done_ops", ctypes.c_int)]


class Optimizer(ctypes.Structure):
    """``nsgb_optimizer`` (include/nsgb.h)."""
    _fields_ = [("kind", ctypes.c_int), ("learning_rate", ctypes.c_double), ("b1", ctypes.c_double),
                ("b2", ctypes.c_double), ("eps", ctypes.c_double), ("eps_root", ctypes.c_double),
                ("decay", ctypes.c_double)]


OPT_SGD, OPT_ADAM, OPT_RMSPROP = 0, 1, 2


class NativeError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_D = ctypes.c_double
_S = ctypes.c_size_t
_PH = ctypes.POINTER(Phys)

SIGNATURES = {
    "nsgb_version": ([], _I),
    "nsgb_last_error": ([], ctypes.c_char_p),
    "nsgb_plan_create": ([_I, _D, ctypes.POINTER(_P)], _I),
    "nsgb_plan_destroy": ([_P], _I),
    "nsgb_plan_set_tiles": ([_P, _I, _I, _I, _I], _I),
    "nsgb_plan_get_tiles": ([_P, ctypes.POINTER(_I)], _I),
    "nsgb_plan_set_fft_radix": ([_P, _I, _I], _I),
    "nsgb_plan_get_fft_radix": ([_P, ctypes.POINTER(_I)], _I),
    "nsgb_plan_set_adjoint_tiles": ([_P, _I, _I], _I),
    "nsgb_plan_get_adjoint_tiles": ([_P, ctypes.POINTER(_I)], _I),
    "nsgb_plan_set_fused": ([_P, _I], _I),
    "nsgb_plan_get_fused": ([_P, ctypes.POINTER(_I)], _I),
    "nsgb_poisson_workspace_bytes": ([_P], _S),
    "nsgb_step_workspace_bytes": ([_P], _S),
    "nsgb_rollout_workspace_bytes": ([_P, _I], _S),
    "nsgb_rollout_grad_workspace_bytes": ([_P, _I, _I], _S),
    "nsgb_grad": ([_P, _P, _P, _P, _P], _I),
    "nsgb_laplacian": ([_P, _P, _P, _P], _I),
    "nsgb_divergence": ([_P, _P, _P, _P], _I),
    "nsgb_advect": ([_P, _I, _P, _P, _P, _P, _P], _I),
    "nsgb_poisson": ([_P, _P, _P, _P, _S, _P], _I),
    "nsgb_forcing": ([_P, _PH, _P, _I, _F, _P, _P], _I),
    "nsgb_projector_step": ([_P, _PH, _P, _P, _P, _P, _S, _P], _I),
    "nsgb_step": ([_P, _PH, _P, _P, _I, _F, _P, _P, _S, _P], _I),
    "nsgb_rollout": ([_P, _PH, _P, _P, _I, _I, _P, _P, _P, _S, _I, _P], _I),
    "nsgb_rollout_grad": ([_P, _PH, _P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _P, _S, _P], _I),
    "nsgb_time_stages": ([_P, _PH, _P, _P, _I, _I, _P, _S, _P, _S, ctypes.POINTER(_F), _P], _I),
    "nsgb_time_step_pipeline": ([_P, _PH, _P, _P, _I, _I, _P, _S, ctypes.POINTER(_F), _P], _I),
    "nsgb_ensemble_workspace_bytes": ([ctypes.POINTER(Member), _I], _S),
    "nsgb_ensemble_advance": ([ctypes.POINTER(Member), _I, _I, _P, _S, _P], _I),
    "nsgb_ensemble_rollout": ([ctypes.POINTER(Member), _I, _I, _P, _S, _P], _I),
    "nsgb_ensemble_persistent_workspace_bytes": ([ctypes.POINTER(Member), _I], _S),
    "nsgb_ensemble_persistent": ([ctypes.POINTER(Member), _I, _P, _S, _P], _I),
    "nsgb_poisson_noalloc": ([_I, _D, _P, _P, _P], _I),
    "nsgb_bounds_checking": ([], _I),
    "nsgb_bounds_register": ([_P, _S], _I),
    "nsgb_bounds_unregister": ([_P], _I),
    "nsgb_bounds_clear": ([], _I),
    "nsgb_grad_ops": ([_I, _I], _I),
    "nsgb_grad_batch_workspace_bytes": ([_I, _I], _S),
    "nsgb_grad_batch_advance": ([ctypes.POINTER(GradMember), _I, _I, _P, _S, _P], _I),
    "nsgb_optimize_workspace_bytes": ([_P, _I, _I, _I], _S),
    "nsgb_optimize": ([_P, _PH, _P, _P, _I, _I, _I, ctypes.POINTER(Optimizer), _I, _P, _P, _P, _S, _P], _I),
}


def lib_path() -> str:
    return _build.LIB


def lib():
    """Load libnsgb.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = lib_path()
            if not os.path.exists(path):
                raise RuntimeError(
                    f"{path} is missing: build the CUDA library first "
                    "(python -m ns_solver_jax_differential_distributed_gb300._build)")
            L = ctypes.CDLL(path)
            for name, (args, res) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = res
            _lib = L
    return _lib


def check(fn: str, status: int) -> None:
    if status != NSGB_OK:
        msg = lib().nsgb_last_error().decode(errors="replace")
        raise NativeError(fn, status, msg)


def call(fn: str, *args):
    check(fn, getattr(lib(), fn)(*args))


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def stream_of(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


# ------------------------------------------------------------------ plans --
class Plan:
    """One ``nsgb_plan`` (constant tables + launch shapes) for (N, L, device)."""

    def __init__(self, N: int, L: float, device: torch.device):
        self.N, self.L, self.device = int(N), float(L), device
        h = _P()
        with torch.cuda.device(device):
            call("nsgb_plan_create", self.N, self.L, ctypes.byref(h))
        self.handle = h
        self._ws: dict = {}

    def tiles(self) -> tuple:
        out = (_I * 4)()
        call("nsgb_plan_get_tiles", self.handle, out)
        return tuple(out)

    def set_tiles(self, tw=0, th=0, rows=0, cols=0) -> None:
        call("nsgb_plan_set_tiles", self.handle, int(tw), int(th), int(rows), int(cols))
        self._ws.clear()

    def fft_radix(self) -> tuple:
        out = (_I * 2)()
        call("nsgb_plan_get_fft_radix", self.handle, out)
        return tuple(out)

    def set_fft_radix(self, rows=0, cols=0) -> None:
        call("nsgb_plan_set_fft_radix", self.handle, int(rows), int(cols))

    def adjoint_tiles(self) -> tuple:
        out = (_I * 2)()
        call("nsgb_plan_get_adjoint_tiles", self.handle, out)
        return tuple(out)

    def set_adjoint_tiles(self, tw=0, th=0) -> None:
        call("nsgb_plan_set_adjoint_tiles", self.handle, int(tw), int(th))

    def fused_rows(self) -> int:
        """Row band of the fused row kernel (0: the four-kernel step)."""
        out = _I()
        call("nsgb_plan_get_fused", self.handle, ctypes.byref(out))
        return int(out.value)

    def set_fused(self, rows: int) -> None:
        """rows > 0: fused row kernel with bands of `rows` rows; -1: the band
        that fits every cluster on the GPU at once; 0: four-kernel step."""
        with torch.cuda.device(self.device):
            call("nsgb_plan_set_fused", self.handle, int(rows))
        self._ws.clear()

    def workspace(self, kind: str, nbytes: int, stream: int) -> torch.Tensor:
        """A cached uint8 workspace of at least nbytes for (kind, stream)."""
        key = (kind, stream)
        ws = self._ws.get(key)
        if ws is None or ws.numel() < nbytes:
            ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.device)
            self._ws[key] = ws
        return ws

    def __del__(self):
        try:
            if getattr(self, "handle", None) and _lib is not None:
                _lib.nsgb_plan_destroy(self.handle)
        except Exception:
            pass


_plans: dict = {}


def get_plan(N: int, L: float, device) -> Plan:
    lib()  # load before taking the plan lock
    device = torch.device(device)
    if device.type != "cuda":
        raise RuntimeError(f"the GB300 solver runs on CUDA devices only, got {device}")
    if device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    key = (int(N), float(L), device.index)
    p = _plans.get(key)
    if p is None:
        with _lock:
            p = _plans.get(key)
            if p is None:
                p = Plan(N, L, device)
                _plans[key] = p
    return p


def make_phys(L, nu, dt, scheme, mu0=0.5, sigma0=0.1, C=1.0) -> Phys:
    sid = SCHEME_IDS.get(scheme, scheme) if isinstance(scheme, str) else int(scheme)
    if isinstance(scheme, str) and scheme not in SCHEME_IDS:
        raise ValueError(f"Unknown advection scheme: '{scheme}'. Choose 'central' or 'upwind'.")
    return Phys(float(L), float(nu), float(dt), float(mu0), float(sigma0), float(C), int(sid))


def _cuda_f32(t: torch.Tensor, name: str) -> torch.Tensor:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if t.device.type != "cuda":
        raise RuntimeError(f"{name} must be a CUDA tensor (no CPU path), got {t.device}")
    if t.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {t.dtype}")
    t = t.contiguous()
    if t.data_ptr() % 16:
        t = t.clone()  # the kernels read fields as aligned float4 groups
    return t


def _square(t: torch.Tensor, name: str, comps: int = 0) -> int:
    shape = tuple(t.shape)
    if comps:
        ok = len(shape) == 3 and shape[0] == comps and shape[1] == shape[2]
    else:
        ok = len(shape) == 2 and shape[0] == shape[1]
    if not ok:
        want = f"({comps}, N, N)" if comps else "(N, N)"
        raise ValueError(f"{name} must have shape {want}, got {shape}")
    return shape[-1]


# ------------------------------------------------------------- torch ops --
@torch.library.custom_op("nsgb::grad", mutates_args=(), device_types="cuda")
def op_grad(f: torch.Tensor, L: float) -> tuple[torch.Tensor, torch.Tensor]:
    f = _cuda_f32(f, "field")
    N = _square(f, "field")
    p = get_plan(N, L, f.device)
    gx, gy = torch.empty_like(f), torch.empty_like(f)
    call("nsgb_grad", p.handle, ptr(f), ptr(gx), ptr(gy), stream_of(f.device))
    return gx, gy


@torch.library.custom_op("nsgb::laplacian", mutates_args=(), device_types="cuda")
def op_laplacian(f: torch.Tensor, L: float) -> torch.Tensor:
    f = _cuda_f32(f, "field")
    N = _square(f, "field")
    p = get_plan(N, L, f.device)
    out = torch.empty_like(f)
    call("nsgb_laplacian", p.handle, ptr(f), ptr(out), stream_of(f.device))
    return out


@torch.library.custom_op("nsgb::divergence", mutates_args=(), device_types="cuda")
def op_divergence(u: torch.Tensor, L: float) -> torch.Tensor:
    u = _cuda_f32(u, "u")
    N = _square(u, "u", 2)
    p = get_plan(N, L, u.device)
    out = torch.empty((N, N), dtype=torch.float32, device=u.device)
    call("nsgb_divergence", p.handle, ptr(u), ptr(out), stream_of(u.device))
    return out


@torch.library.custom_op("nsgb::advect", mutates_args=(), device_types="cuda")
def op_advect(field: torch.Tensor, ux: torch.Tensor, uy: torch.Tensor, L: float,
              scheme: int) -> torch.Tensor:
    field, ux, uy = (_cuda_f32(field, "field"), _cuda_f32(ux, "ux"), _cuda_f32(uy, "uy"))
    N = _square(field, "field")
    if ux.shape != field.shape or uy.shape != field.shape:
        raise ValueError("field, ux and uy must have the same (N, N) shape")
    p = get_plan(N, L, field.device)
    out = torch.empty_like(field)
    call("nsgb_advect", p.handle, int(scheme), ptr(field), ptr(ux), ptr(uy), ptr(out),
         stream_of(field.device))
    return out


@torch.library.custom_op("nsgb::poisson", mutates_args=(), device_types="cuda")
def op_poisson(rhs: torch.Tensor, L: float) -> torch.Tensor:
    rhs = _cuda_f32(rhs, "rhs")
    N = _square(rhs, "rhs")
    p = get_plan(N, L, rhs.device)
    st = stream_of(rhs.device)
    nbytes = lib().nsgb_poisson_workspace_bytes(p.handle)
    ws = p.workspace("poisson", nbytes, st)
    out = torch.empty_like(rhs)
    call("nsgb_poisson", p.handle, ptr(rhs), ptr(out), ptr(ws), ws.numel(), st)
    return out


@torch.library.custom_op("nsgb::forcing", mutates_args=(), device_types="cuda")
def op_forcing(theta: torch.Tensor, t: float, N: int, L: float, mu0: float, sigma0: float,
               C: float) -> torch.Tensor:
    theta = _cuda_f32(theta, "theta")
    p = get_plan(N, L, theta.device)
    ph = make_phys(L, 1.0, 1.0, 0, mu0, sigma0, C)
    out = torch.empty((2, N, N), dtype=torch.float32, device=theta.device)
    call("nsgb_forcing", p.handle, ctypes.byref(ph), ptr(theta), theta.numel(), float(t), ptr(out),
         stream_of(theta.device))
    return out


@torch.library.custom_op("nsgb::projector_step", mutates_args=(), device_types="cuda")
def op_projector_step(u: torch.Tensor, f: torch.Tensor, L: float, nu: float, dt: float,
                      scheme: int) -> torch.Tensor:
    u, f = _cuda_f32(u, "u"), _cuda_f32(f, "f")
    N = _square(u, "u", 2)
    _square(f, "f", 2)
    p = get_plan(N, L, u.device)
    st = stream_of(u.device)
    ph = make_phys(L, nu, dt, scheme)
    ws = p.workspace("step", lib().nsgb_step_workspace_bytes(p.handle), st)
    out = torch.empty_like(u)
    call("nsgb_projector_step", p.handle, ctypes.byref(ph), ptr(u), ptr(f), ptr(out), ptr(ws),
         ws.numel(), st)
    return out


@torch.library.custom_op("nsgb::step", mutates_args=(), device_types="cuda")
def op_step(u: torch.Tensor, theta: torch.Tensor, t: float, L: float, nu: float, dt: float,
            scheme: int, mu0: float, sigma0: float, C: float) -> torch.Tensor:
    u, theta = _cuda_f32(u, "u"), _cuda_f32(theta, "theta")
    N = _square(u, "u", 2)
    p = get_plan(N, L, u.device)
    st = stream_of(u.device)
    ph = make_phys(L, nu, dt, scheme, mu0, sigma0, C)
    ws = p.workspace("step", lib().nsgb_step_workspace_bytes(p.handle), st)
    out = torch.empty_like(u)
    call("nsgb_step", p.handle, ctypes.byref(ph), ptr(u), ptr(theta), theta.numel(), float(t),
         ptr(out), ptr(ws), ws.numel(), st)
    return out


@torch.library.custom_op("nsgb::rollout", mutates_args=(), device_types="cuda")
def op_rollout(u0: torch.Tensor, theta: torch.Tensor, steps: int, L: float, nu: float, dt: float,
               scheme: int, mu0: float, sigma0: float, C: float,
               use_graph: bool) -> tuple[torch.Tensor, torch.Tensor]:
    u0, theta = _cuda_f32(u0, "u0"), _cuda_f32(theta, "theta")
    N = _square(u0, "u0", 2)
    p = get_plan(N, L, u0.device)
    st = stream_of(u0.device)
    ph = make_phys(L, nu, dt, scheme, mu0, sigma0, C)
    nbytes = lib().nsgb_rollout_workspace_bytes(p.handle, int(steps))
    ws = p.workspace("rollout", nbytes, st)
    J = torch.empty((), dtype=torch.float32, device=u0.device)
    uf = torch.empty_like(u0)
    call("nsgb_rollout", p.handle, ctypes.byref(ph), ptr(u0), ptr(theta), theta.numel(), int(steps),
         ptr(uf), ptr(J), ptr(ws), ws.numel(), int(bool(use_graph)), st)
    return J, uf


def rollout_grad_raw(u0: torch.Tensor, theta: torch.Tensor, steps: int, every: int, L: float,
                     nu: float, dt: float, scheme, mu0=0.5, sigma0=0.1, C=1.0,
                     want_u_final: bool = True, want_du0: bool = False, own_workspace: bool = False):
    """Forward + adjoint in one call: returns (J, dJ/dtheta, u_final, dJ/du0).
    With own_workspace the scratch is allocated for this call only (freed when
    the call's tensors are), instead of the plan's cached workspace."""
    u0, theta = _cuda_f32(u0, "u0"), _cuda_f32(theta, "theta")
    N = _square(u0, "u0", 2)
    p = get_plan(N, L, u0.device)
    st = stream_of(u0.device)
    ph = make_phys(L, nu, dt, scheme, mu0, sigma0, C)
    nbytes = lib().nsgb_rollout_grad_workspace_bytes(p.handle, int(steps), int(every))
    if own_workspace:
        ws = torch.empty(nbytes, dtype=torch.uint8, device=u0.device)
    else:
        ws = p.workspace("grad", nbytes, st)
    J = torch.empty((), dtype=torch.float32, device=u0.device)
    g = torch.empty(theta.numel(), dtype=torch.float32, device=u0.device)
    uf = torch.empty_like(u0) if want_u_final else None
    du0 = torch.empty_like(u0) if want_du0 else None
    call("nsgb_rollout_grad", p.handle, ctypes.byref(ph), ptr(u0), ptr(theta), theta.numel(),
         int(steps), int(every), GRAD_FORWARD | GRAD_BACKWARD, ptr(J), ptr(uf), ptr(g), ptr(du0),
         ptr(ws), ws.numel(), st)
    return J, g, uf, du0


class GradSession:
    """Workspace of one differentiable rollout: the forward phase keeps the
    checkpoints on the device for the backward phase."""

    def __init__(self, u0, theta, steps, every, L, nu, dt, scheme, mu0=0.5, sigma0=0.1, C=1.0):
        self.u0 = _cuda_f32(u0, "u0")
        self.theta = _cuda_f32(theta, "theta")
        self.N = _square(self.u0, "u0", 2)
        self.plan = get_plan(self.N, L, self.u0.device)
        self.steps, self.every = int(steps), int(every)
        self.ph = make_phys(L, nu, dt, scheme, mu0, sigma0, C)
        nbytes = lib().nsgb_rollout_grad_workspace_bytes(self.plan.handle, self.steps, self.every)
        # Owned by the session (not the plan's cache): it must outlive forward().
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.u0.device)

    def forward(self):
        st = stream_of(self.u0.device)
        J = torch.empty((), dtype=torch.float32, device=self.u0.device)
        uf = torch.empty_like(self.u0)
        call("nsgb_rollout_grad", self.plan.handle, ctypes.byref(self.ph), ptr(self.u0),
             ptr(self.theta), self.theta.numel(), self.steps, self.every, GRAD_FORWARD, ptr(J),
             ptr(uf), None, None, ptr(self.ws), self.ws.numel(), st)
        return J, uf

    def backward(self, want_du0: bool = True):
        st = stream_of(self.u0.device)
        g = torch.empty(self.theta.numel(), dtype=torch.float32, device=self.u0.device)
        du0 = torch.empty_like(self.u0) if want_du0 else None
        call("nsgb_rollout_grad", self.plan.handle, ctypes.byref(self.ph), ptr(self.u0),
             ptr(self.theta), self.theta.numel(), self.steps, self.every, GRAD_BACKWARD, None,
             None, ptr(g), ptr(du0), ptr(self.ws), self.ws.numel(), st)
        return g, du0


STAGES = ("stencil", "rows_fwd", "cols", "rows_inv")
FUSED_STAGES = ("fused", "cols")
# Algorithmic bytes per cell of each stage (float32): stencil reads u* (8) and
# p (4) and writes u* (8) and rhs (4); each FFT pass reads and writes the
# half spectrum or the real field once (4 + 4); the fused row kernel reads u*
# (8) and the solved half spectrum (4) and writes u* (8) and the new half
# spectrum (4).
STAGE_BYTES_PER_CELL = {"stencil": 24, "rows_fwd": 8, "cols": 8, "rows_inv": 8, "fused": 24}


def _stage_dict(p: "Plan", out) -> dict:
    if p.fused_rows() > 0:
        return {"fused": float(out[0]), "cols": float(out[1])}
    return dict(zip(STAGES, [float(x) for x in out]))


def time_stages(u0: torch.Tensor, theta: torch.Tensor, L: float, nu: float, dt: float, scheme,
                reps: int = 20, flush: torch.Tensor | None = None) -> dict:
    """Mean device ms per launch of each stage kernel (CUDA events, cold L2
    when `flush` is given)."""
    u0, theta = _cuda_f32(u0, "u0"), _cuda_f32(theta, "theta")
    N = _square(u0, "u0", 2)
    p = get_plan(N, L, u0.device)
    st = stream_of(u0.device)
    ph = make_phys(L, nu, dt, scheme)
    ws = p.workspace("time", lib().nsgb_rollout_workspace_bytes(p.handle, 1), st)
    out = (_F * 4)()
    call("nsgb_time_stages", p.handle, ctypes.byref(ph), ptr(u0), ptr(theta), theta.numel(), int(reps),
         ptr(flush), 0 if flush is None else flush.numel() * flush.element_size(), ptr(ws), ws.numel(),
         out, st)
    return _stage_dict(p, out)


def time_step_pipeline(u0: torch.Tensor, theta: torch.Tensor, L: float, nu: float, dt: float, scheme,
                       steps: int = 20) -> dict:
    """Mean device ms per launch of each stage kernel inside `steps`
    back-to-back solver steps (CUDA events between consecutive kernels, L2
    shared between them as in a rollout)."""
    u0, theta = _cuda_f32(u0, "u0"), _cuda_f32(theta, "theta")
    N = _square(u0, "u0", 2)
    p = get_plan(N, L, u0.device)
    st = stream_of(u0.device)
    ph = make_phys(L, nu, dt, scheme)
    ws = p.workspace("time_pipe", lib().nsgb_rollout_workspace_bytes(p.handle, int(steps) + 1), st)
    out = (_F * 4)()
    call("nsgb_time_step_pipeline", p.handle, ctypes.byref(ph), ptr(u0), ptr(theta), theta.numel(), int(steps),
         ptr(ws), ws.numel(), out, st)
    return _stage_dict(p, out)


def optimize(theta0: torch.Tensor, steps: int, every: int, N: int, L: float, nu: float, dt: float, scheme,
             opt: Optimizer, iters: int, u0: torch.Tensor | None = None, mu0=0.5, sigma0=0.1, C=1.0):
    """nsgb_optimize: `iters` optimiser steps on the device from theta0 (zero
    initial state when u0 is None).  Returns (objectives[iters+1],
    parameters[iters+1, len(theta0)]) as device tensors."""
    theta0 = _cuda_f32(theta0, "theta0")
    dev = theta0.device
    if u0 is not None:
        u0 = _cuda_f32(u0, "u0")
        if _square(u0, "u0", 2) != N:
            raise ValueError(f"u0 must be (2, {N}, {N})")
    p = get_plan(N, L, dev)
    st = stream_of(dev)
    ph = make_phys(L, nu, dt, scheme, mu0, sigma0, C)
    n = theta0.numel()
    nbytes = lib().nsgb_optimize_workspace_bytes(p.handle, int(steps), int(every), n)
    if nbytes == 0:
        raise ValueError("invalid optimisation arguments (steps >= 1, every >= 1, theta of 2 or 3 entries)")
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    objectives = torch.empty(iters + 1, dtype=torch.float32, device=dev)
    parameters = torch.empty(iters + 1, n, dtype=torch.float32, device=dev)
    call("nsgb_optimize", p.handle, ctypes.byref(ph), ptr(u0), ptr(theta0), n, int(steps), int(every),
         ctypes.byref(opt), int(iters), ptr(objectives), ptr(parameters), ptr(ws), ws.numel(), st)
    return objectives, parameters
