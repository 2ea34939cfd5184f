"""Reference-compatible API of the single-device Chorin-projection solver.

Mirrors the public surface of ``NS_solver.py`` of
helmhlotz/ns_solver_jax_differential_distributed (same class names,
constructor arguments, method names and error behaviour), with torch CUDA
tensors in place of JAX arrays.  Every numerical method runs hand-written
sm_103a CUDA kernels through the C ABI (``include/nsgb.h``); there is no CPU
path.  Inputs may be CPU tensors, NumPy arrays or lists: they are copied to the
solver's CUDA device, and results are returned as CUDA tensors.
"""
from __future__ import annotations

import json
import logging
import math
import os
from dataclasses import dataclass, field
from typing import Optional, Tuple

import numpy as np
import torch

from . import _native

logger = logging.getLogger(__name__)


def setup_logger(name: str, level: int = logging.INFO) -> logging.Logger:
    """Stream logger with the reference's '[name] LEVEL: msg' format (NS_solver.py:21-29)."""
    lg = logging.getLogger(name)
    lg.setLevel(level)
    lg.handlers = []
    h = logging.StreamHandler()
    h.setLevel(level)
    h.setFormatter(logging.Formatter('[%(name)s] %(levelname)s: %(message)s'))
    lg.addHandler(h)
    return lg


def _device(device=None) -> torch.device:
    if device is not None:
        return torch.device(device)
    if not torch.cuda.is_available():
        raise RuntimeError("the GB300 solver needs a CUDA device (there is no CPU path)")
    return torch.device("cuda", torch.cuda.current_device())


def _as_f32(x, device: torch.device) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float32).contiguous()
    return torch.as_tensor(np.asarray(x, dtype=np.float32), device=device).contiguous()


# ============================================================ configuration
@dataclass(frozen=True)
class SimConfig:
    """Centralized simulation configuration (NS_solver.py:41-79)."""
    N: int = 128
    L: float = 1.0
    nu: float = 0.01
    mu0: float = 0.5
    sigma0: float = 0.1
    C_force: float = 1.0
    cfl: float = 0.4
    v_max: float = 1.0
    t: float = 0.5
    theta0: Optional[object] = None
    advection_scheme: str = "central"
    obj_tol: float = 1e-6

    def __post_init__(self):
        # Validation of NS_solver.py:56-64.
        if self.N <= 0:
            raise ValueError(f"Grid resolution N must be positive, got {self.N}")
        if self.nu <= 0:
            raise ValueError(f"Kinematic viscosity nu must be positive, got {self.nu}")
        if self.advection_scheme not in ("central", "upwind"):
            raise ValueError(
                f"Advection scheme must be 'central' or 'upwind', got {self.advection_scheme}")
        if self.theta0 is None:
            object.__setattr__(self, "theta0", np.array([1.0, 0.5], dtype=np.float32))
        else:
            object.__setattr__(self, "theta0", np.asarray(self.theta0, dtype=np.float32))

    @property
    def steps(self) -> int:
        return int(np.ceil(self.t / self.dt))

    @property
    def dx(self) -> float:
        return self.L / self.N

    @property
    def dt(self) -> float:
        """Stable step: min of the CFL and diffusive limits, rounded through
        float32 as ``float(jnp.minimum(...))`` does (NS_solver.py:75-79)."""
        dt_adv = self.cfl * self.dx / self.v_max
        dt_diff = (self.dx ** 2) / (4.0 * self.nu)
        return float(np.float32(min(dt_adv, dt_diff)))


@dataclass(frozen=True)
class Grid:
    """Uniform periodic grid on [0, L]^2 (NS_solver.py:90-92)."""
    N: int
    L: float
    dx: float
    X: torch.Tensor = field(repr=False)
    Y: torch.Tensor = field(repr=False)


@dataclass(frozen=True)
class Phys:
    """Physical parameters (NS_solver.py:99-101)."""
    nu: float
    mu0: float
    sigma0: float
    C: float


@dataclass(frozen=True)
class Time:
    """Time integration parameters (NS_solver.py:108-110)."""
    dt: float
    steps: int


def make_grid(N: int, L: float = 1.0, device=None) -> Grid:
    """Grid with X, Y = meshgrid(linspace(0, L, N, endpoint=False)) in float32
    (NS_solver.py:112-117).  X and Y are kept on the host unless a device is
    given: the kernels evaluate x_i = L * (i/N) themselves."""
    dx = L / N
    s = (np.arange(N, dtype=np.float32) / np.float32(N)).astype(np.float32)
    x = (np.float32(L) * s).astype(np.float32)
    X, Y = np.meshgrid(x, x, indexing="ij")
    X, Y = torch.from_numpy(X), torch.from_numpy(Y)
    if device is not None:
        X, Y = X.to(device), Y.to(device)
    return Grid(N, L, dx, X, Y)


def load_config(path: Optional[str] = None) -> SimConfig:
    """Load a SimConfig from JSON, defaults for missing fields, unknown fields
    ignored with a warning, theta0 read separately (NS_solver.py:120-172)."""
    defaults = {f: getattr(SimConfig(), f) for f in SimConfig.__dataclass_fields__ if f != "theta0"}
    if path is None:
        logger.info("No config file specified -- using default SimConfig.")
        return SimConfig()
    if not os.path.exists(path):
        logger.warning(f"Config file not found: '{path}' -- using default SimConfig.")
        return SimConfig()
    with open(path, "r") as f:
        user = json.load(f)
    unknown = set(user) - set(defaults) - {"theta0"}
    if unknown:
        logger.warning(f"Ignoring unrecognised config fields: {unknown}")
    merged = {**defaults, **{k: v for k, v in user.items() if k in defaults}}
    theta0 = np.asarray(user["theta0"], dtype=np.float32) if "theta0" in user else None
    cfg = SimConfig(**merged, theta0=theta0)
    logger.info(f"Loaded config from '{path}': N={cfg.N}, nu={cfg.nu}, "
                f"scheme={cfg.advection_scheme}, time={cfg.t}, steps={cfg.steps}, dt={cfg.dt:.6e}")
    return cfg


CONFIG = SimConfig()


# ==================================================== differential operators
class DifferentialOps:
    """Interface of the spatial operators on a periodic grid (NS_solver.py:186-234)."""

    def __init__(self, dx: float):
        self.dx = dx

    def grad(self, field: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
        raise NotImplementedError

    def laplacian(self, field: torch.Tensor) -> torch.Tensor:
        raise NotImplementedError

    def divergence(self, u: torch.Tensor) -> torch.Tensor:
        gx, _ = self.grad(u[0])
        _, gy = self.grad(u[1])
        return gx + gy

    def upwind_advect(self, field, ux, uy) -> torch.Tensor:
        raise NotImplementedError

    def divergence_vec(self, u: torch.Tensor) -> torch.Tensor:
        return self.divergence(u)

    def laplacian_and_advect_vec(self, u: torch.Tensor, advection: "AdvectionScheme"):
        ux, uy = u[0], u[1]
        lap = torch.stack([self.laplacian(ux), self.laplacian(uy)], dim=0)
        adv = torch.stack([advection.advect(ux, ux, uy, self), advection.advect(uy, ux, uy, self)],
                          dim=0)
        return lap, adv


class PeriodicDifferentialOps(DifferentialOps):
    """Single-device periodic stencils (NS_solver.py:237-265), each a CUDA kernel."""

    def _L(self, field: torch.Tensor) -> float:
        return self.dx * field.shape[-1]

    def grad(self, field):
        return _native.op_grad(field, self._L(field))

    def laplacian(self, field):
        return _native.op_laplacian(field, self._L(field))

    def divergence(self, u):
        return _native.op_divergence(u, self._L(u))

    def upwind_advect(self, field, ux, uy):
        return _native.op_advect(field, ux, uy, self._L(field), 1)

    def central_advect(self, field, ux, uy):
        return _native.op_advect(field, ux, uy, self._L(field), 0)


# ========================================================= advection schemes
class AdvectionScheme:
    """Interface of -(u.grad)phi discretisations (NS_solver.py:450-465)."""
    name = ""

    def advect(self, field, ux, uy, ops: DifferentialOps):
        raise NotImplementedError


class CentralAdvection(AdvectionScheme):
    """-(ux dphi/dx + uy dphi/dy) with central differences (NS_solver.py:468-477)."""
    name = "central"

    def advect(self, field, ux, uy, ops):
        if type(ops) is PeriodicDifferentialOps:
            return ops.central_advect(field, ux, uy)
        fx, fy = ops.grad(field)
        return -(ux * fx + uy * fy)


class UpwindAdvection(AdvectionScheme):
    """First-order upwind differences (NS_solver.py:480-488)."""
    name = "upwind"

    def advect(self, field, ux, uy, ops):
        return ops.upwind_advect(field, ux, uy)


def make_advection_scheme(name: str) -> AdvectionScheme:
    """Factory (NS_solver.py:491-497)."""
    if name == "central":
        return CentralAdvection()
    elif name == "upwind":
        return UpwindAdvection()
    raise ValueError(f"Unknown advection scheme: '{name}'. Choose 'central' or 'upwind'.")


# ============================================================ Poisson solver
class SpectralPoissonSolver:
    """Spectral pressure solve p = Re ifft2(-fft2(rhs) / |k|^2), p_hat[0,0] = 0,
    i.e. lap(p) = rhs (NS_solver.py:507-527), by hand-written R2C/C2R FFTs."""

    def __init__(self, Nx: int, Ny: int, dx: float):
        if Nx != Ny:
            raise ValueError(f"the GB300 solver needs a square grid, got {Nx} x {Ny}")
        self.Nx, self.Ny, self.dx = Nx, Ny, dx
        self.L = dx * Nx

    @property
    def _inv_k2(self) -> torch.Tensor:
        """1/|k|^2 with the (0,0) entry zeroed, float32 (NS_solver.py:518-521)."""
        N, dx = self.Nx, self.dx
        m = np.concatenate([np.arange(0, N // 2), np.arange(-(N // 2), 0)]).astype(np.float32)
        k = ((m / np.float32(dx * N)).astype(np.float32) * np.float32(2)).astype(np.float32)
        k = (k * np.float32(np.pi)).astype(np.float32)
        KX, KY = np.meshgrid(k, k, indexing="ij")
        k2 = (KX * KX + KY * KY).astype(np.float32)
        with np.errstate(divide="ignore"):
            inv = np.where(k2 == 0, np.float32(0), np.float32(1) / k2).astype(np.float32)
        return torch.from_numpy(inv)

    def __call__(self, rhs: torch.Tensor) -> torch.Tensor:
        return _native.op_poisson(rhs, self.L)


# ================================================================== forcing
class GaussianForcingField:
    """f = (C exp(-d(x, mu(t))^2 / 2 sigma(t)^2), 0) with mu = mu0 + sin(2 pi A t),
    sigma = sigma0 + cos^2(2 pi B t) and d wrapped with period 1
    (NS_solver.py:606-640)."""

    def __init__(self, grid: Grid, phys: Phys):
        self.grid = grid
        self.phys = phys

    def _x_component(self, theta, t, x):
        """Profile at the given x-coordinates (NS_solver.py:621-627), float32
        torch arithmetic on x's device."""
        th = torch.as_tensor(theta, dtype=torch.float32, device=x.device)
        A, B = th[0], th[1]
        t = torch.tensor(float(t), dtype=torch.float32, device=x.device)
        twopi = torch.tensor(2.0 * math.pi, dtype=torch.float32, device=x.device)
        mu = self.phys.mu0 + torch.sin(twopi * A * t)
        c = torch.cos(twopi * B * t)
        sig = self.phys.sigma0 + c * c
        d = (x - mu) - torch.round(x - mu)
        return self.phys.C * torch.exp(-(d * d) / (2.0 * sig * sig))

    def __call__(self, theta, t: float) -> torch.Tensor:
        dev = theta.device if isinstance(theta, torch.Tensor) and theta.is_cuda else _device()
        th = _as_f32(theta, dev)
        return _native.op_forcing(th, float(t), self.grid.N, float(self.grid.L), float(self.phys.mu0),
                                  float(self.phys.sigma0), float(self.phys.C))


# ========================================================== Chorin projector
class ChorinProjector:
    """One explicit-Euler + pressure-projection step (NS_solver.py:654-697).

    With the standard strategies (PeriodicDifferentialOps, SpectralPoissonSolver,
    Central/UpwindAdvection) a step is one fused stencil kernel, the FFT-Poisson
    kernels and a projection kernel.  Other strategy objects are composed
    through their own methods, as the reference does.
    """

    def __init__(self, ops: DifferentialOps, poisson: SpectralPoissonSolver,
                 advection: AdvectionScheme, nu: float, dt: float):
        self.ops = ops
        self.poisson = poisson
        self.advection = advection
        self.nu = nu
        self.dt = dt

    def _fused(self) -> bool:
        return (type(self.ops) is PeriodicDifferentialOps
                and type(self.poisson) is SpectralPoissonSolver
                and type(self.advection) in (CentralAdvection, UpwindAdvection))

    def step(self, u: torch.Tensor, f: torch.Tensor) -> torch.Tensor:
        if self._fused():
            L = self.ops.dx * u.shape[-1]
            sid = _native.SCHEME_IDS[self.advection.name]
            return _native.op_projector_step(u, f, L, float(self.nu), float(self.dt), sid)
        ux, uy = u[0], u[1]
        ops, dt, nu = self.ops, self.dt, self.nu
        lap_u, adv_u = ops.laplacian_and_advect_vec(u, self.advection)
        ux_star = ux + dt * (nu * lap_u[0] + adv_u[0] + f[0])
        uy_star = uy + dt * (nu * lap_u[1] + adv_u[1] + f[1])
        u_star = torch.stack([ux_star, uy_star], dim=0)
        div_star = ops.divergence_vec(u_star)
        p = self.poisson(div_star / dt)
        px, py = ops.grad(p)
        return torch.stack([ux_star - dt * px, uy_star - dt * py], dim=0)


# ================================================================== solvers
class _RolloutFn(torch.autograd.Function):
    """Differentiable rollout: forward keeps checkpoints on the device, backward
    runs the hand-written discrete adjoint (dJ/dtheta and dJ/du0)."""

    @staticmethod
    def forward(ctx, theta, u0, solver, every):
        sess = _native.GradSession(u0.detach(), theta.detach(), solver.time.steps, every,
                                   solver.grid.L, solver.phys.nu, solver.time.dt,
                                   solver.advection_scheme, solver.phys.mu0, solver.phys.sigma0,
                                   solver.phys.C)
        J, uf = sess.forward()
        ctx.sess = sess
        ctx.mark_non_differentiable(uf)
        return J, uf

    @staticmethod
    def backward(ctx, gJ, guf):
        g, du0 = ctx.sess.backward(want_du0=ctx.needs_input_grad[1])
        ctx.sess = None
        gtheta = g * gJ
        gu0 = du0 * gJ if du0 is not None else None
        return gtheta, gu0, None, None


class SingleCoreNSSolver:
    """Single-device solver (NS_solver.py:707-756): step, rollout, objective,
    jit_objective and jit_gradient, on the GB300 kernels.

    ``theta`` may hold 2 entries [A, B] (the reference) or 3 entries
    [A, B, nu], where the third replaces the viscosity.
    """

    def __init__(self, grid: Grid, phys: Phys, time_cfg: Time, advection_scheme: str = "central",
                 device=None, checkpoint_every: Optional[int] = None, use_graph: bool = True):
        self.grid = grid
        self.time = time_cfg
        self.phys = phys
        self.device = _device(device)
        self.advection_scheme = advection_scheme
        ops = PeriodicDifferentialOps(grid.dx)
        poisson = SpectralPoissonSolver(grid.N, grid.N, grid.dx)
        advection = make_advection_scheme(advection_scheme)
        self.forcing = GaussianForcingField(grid, phys)
        self.projector = ChorinProjector(ops, poisson, advection, phys.nu, time_cfg.dt)
        # None: store every state when they fit in half the free device memory
        # (no recomputation in the backward pass), else checkpoints every
        # ceil(sqrt(steps)) steps
        self.checkpoint_every = None if checkpoint_every is None else int(checkpoint_every)
        self.use_graph = bool(use_graph)
        self._scheme_id = _native.SCHEME_IDS[advection_scheme]
        self.jit_objective = self.objective
        self.jit_gradient = self.gradient_zero_ic

    # -- helpers
    def _every(self) -> int:
        if self.checkpoint_every is not None:
            return self.checkpoint_every
        steps = int(self.time.steps)
        state = 8 * self.grid.N * self.grid.N
        free, _ = torch.cuda.mem_get_info(self.device)
        if (steps + 1) * state <= free // 2:
            return 1
        return max(1, math.isqrt(max(steps - 1, 0)) + 1)

    def _theta(self, theta) -> torch.Tensor:
        th = _as_f32(theta, self.device).reshape(-1)
        if th.numel() not in (2, 3):
            raise ValueError(f"theta must have 2 or 3 entries, got {th.numel()}")
        return th

    def _u(self, u) -> torch.Tensor:
        u = _as_f32(u, self.device)
        N = self.grid.N
        if tuple(u.shape) != (2, N, N):
            raise ValueError(f"u must have shape (2, {N}, {N}), got {tuple(u.shape)}")
        return u

    # -- reference API
    def step(self, u, theta, t: float) -> torch.Tensor:
        """One step with the Gaussian forcing at time t (NS_solver.py:727-730)."""
        g, ph = self.grid, self.phys
        return _native.op_step(self._u(u), self._theta(theta), float(t), float(g.L), float(ph.nu),
                               float(self.time.dt), self._scheme_id, float(ph.mu0),
                               float(ph.sigma0), float(ph.C))

    def rollout(self, u0, theta) -> Tuple[torch.Tensor, torch.Tensor]:
        """Integrate time.steps steps from u0 and return (J, u_final) with
        J = sum_t dt * sum(u(t) * f(t)) * dx^2 on the state before each step
        (NS_solver.py:732-750).  Differentiable in theta and u0 through the
        hand-written adjoint when either requires grad."""
        th = self._theta(theta) if not isinstance(theta, torch.Tensor) else theta
        u0t = self._u(u0) if not isinstance(u0, torch.Tensor) else u0
        if torch.is_grad_enabled() and (
                (isinstance(th, torch.Tensor) and th.requires_grad) or
                (isinstance(u0t, torch.Tensor) and u0t.requires_grad)):
            th_d = th.to(self.device, torch.float32).reshape(-1)
            u0_d = u0t.to(self.device, torch.float32)
            # the same checks as the plain path (the session would otherwise
            # take N from u0)
            if th_d.numel() not in (2, 3):
                raise ValueError(f"theta must have 2 or 3 entries, got {th_d.numel()}")
            N = self.grid.N
            if tuple(u0_d.shape) != (2, N, N):
                raise ValueError(f"u must have shape (2, {N}, {N}), got {tuple(u0_d.shape)}")
            return _RolloutFn.apply(th_d, u0_d, self, self._every())
        th = self._theta(th)
        u0t = self._u(u0t)
        g, ph = self.grid, self.phys
        return _native.op_rollout(u0t, th, int(self.time.steps), float(g.L), float(ph.nu),
                                  float(self.time.dt), self._scheme_id, float(ph.mu0),
                                  float(ph.sigma0), float(ph.C), self.use_graph)

    def objective(self, theta) -> torch.Tensor:
        """J(theta) from a zero initial condition (NS_solver.py:752-756)."""
        u0 = torch.zeros((2, self.grid.N, self.grid.N), dtype=torch.float32, device=self.device)
        J, _ = self.rollout(u0, theta)
        return J

    def gradient(self, u0, theta, want_u0_grad: bool = False):
        """dJ/dtheta of rollout(u0, theta) by the discrete adjoint with
        checkpoints every ``checkpoint_every`` steps (every state when None
        and they fit).  Returns (J, dJ/dtheta) or (J, dJ/dtheta, dJ/du0)."""
        g, ph = self.grid, self.phys
        J, gt, _, du0 = _native.rollout_grad_raw(
            self._u(u0), self._theta(theta), int(self.time.steps), self._every(),
            float(g.L), float(ph.nu), float(self.time.dt), self._scheme_id, float(ph.mu0),
            float(ph.sigma0), float(ph.C), want_u_final=False, want_du0=want_u0_grad)
        return (J, gt, du0) if want_u0_grad else (J, gt)

    def gradient_zero_ic(self, theta) -> torch.Tensor:
        """jax.jit(jax.grad(objective)) of the reference (NS_solver.py:725)."""
        u0 = torch.zeros((2, self.grid.N, self.grid.N), dtype=torch.float32, device=self.device)
        return self.gradient(u0, theta)[1]
