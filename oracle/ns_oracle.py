"""CPU oracle for the single-device Chorin projection step (TEST INFRASTRUCTURE).

This module is the correctness checker of the GB300 solver, nothing more: only
the tests, the smoke check and the CPU-baseline leg of the benchmark may import
it.  The product path never calls into it, and it has no GPU code.

It restates, line for line, the numerical algorithm of the reference JAX
solver (``NS_solver.py`` of helmhlotz/ns_solver_jax_differential_distributed)
in NumPy, in two precisions:

* ``float32`` -- mirrors the reference's default JAX dtype: every array op is
  evaluated in float32 and the FFTs are complex64 C2C transforms, as
  ``jnp.fft.fft2`` performs on a real float32 field.
* ``float64`` -- the same algorithm in double precision (the reference with
  ``jax_enable_x64``), used to state the error of the float32 paths.

Parity pin: the reference cannot run here (JAX is not installed), so this
restatement is pinned against the reference's own shipped outputs
(``result/*.npz`` objectives, kinetic energies, the SGD trajectory of the
optimisation study, and the ``result/velocity_magnitude_*.npy`` speed fields);
``tests/golden/make_golden.py`` extracts them and ``tests/test_oracle_golden.py``
checks this module against them.

Each function cites the reference line it restates.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

__all__ = [
    "OracleConfig", "grid_x", "poisson_inv_k2", "forcing_fx", "grad", "laplacian",
    "divergence", "upwind_advect", "central_advect", "poisson_solve",
    "projector_step", "solver_step", "rollout", "objective", "fd_gradient", "set_fft_workers",
]


@dataclass(frozen=True)
class OracleConfig:
    """Static parameters of one solve (reference ``Grid``/``Phys``/``Time``,
    NS_solver.py:90-110).  ``nu`` may be overridden by a third theta entry."""
    N: int
    L: float
    nu: float
    dt: float
    steps: int
    scheme: str = "central"
    mu0: float = 0.5
    sigma0: float = 0.1
    C: float = 1.0

    @property
    def dx(self) -> float:
        # NS_solver.py:114 (dx = L / N, a Python float)
        return self.L / self.N


def _c(x, dtype):
    """A Python scalar as the dtype the reference's weak typing gives it."""
    return dtype(x)


def grid_x(N: int, L: float, dtype=np.float32) -> np.ndarray:
    """x-coordinates of the grid rows.

    NS_solver.py:115 uses ``jnp.linspace(0, L, N, endpoint=False)``, which JAX
    evaluates as ``start*(1-s) + stop*s`` with ``s = iota/N`` in the array
    dtype; with start = 0 that is ``fl(L * fl(i / N))``.
    """
    s = (np.arange(N, dtype=dtype) / dtype(N)).astype(dtype)
    return (dtype(0.0) * (dtype(1.0) - s) + dtype(L) * s).astype(dtype)


def poisson_inv_k2(N: int, dx: float, dtype=np.float32) -> np.ndarray:
    """1/|k|^2 with the (0,0) entry zeroed (NS_solver.py:517-521).

    ``k = fftfreq(N, d=dx) * 2 * pi``: fftfreq returns integer frequencies
    divided by ``d*N`` in the array dtype; the Nyquist entry is negative.
    """
    m = np.concatenate([np.arange(0, N // 2), np.arange(-(N // 2), 0)]).astype(dtype)
    k = (m / dtype(dx * N)).astype(dtype)
    k = (k * dtype(2)).astype(dtype) * dtype(np.pi)
    k = k.astype(dtype)
    KX, KY = np.meshgrid(k, k, indexing="ij")
    k2 = (KX * KX + KY * KY).astype(dtype)
    with np.errstate(divide="ignore"):
        inv = np.where(k2 == 0, dtype(0.0), dtype(1.0) / k2).astype(dtype)
    return inv


def forcing_fx(theta, t, cfg: OracleConfig, dtype=np.float32) -> np.ndarray:
    """x-component of the Gaussian forcing at the N grid rows (NS_solver.py:621-627).

    mu = mu0 + sin(2*pi*A*t); sigma = sigma0 + cos(2*pi*B*t)**2;
    d = (x - mu) - round(x - mu)   (period 1, round half to even);
    fx = C * exp(-(d*d) / (2*sigma*sigma)).
    """
    th = np.asarray(theta, dtype=dtype)
    A, B = th[0], th[1]
    t = dtype(t)
    twopi = dtype(2.0 * math.pi)
    mu = dtype(cfg.mu0) + np.sin(twopi * A * t, dtype=dtype)
    c = np.cos(twopi * B * t, dtype=dtype)
    sig = dtype(cfg.sigma0) + c * c
    x = grid_x(cfg.N, cfg.L, dtype)
    r = (x - mu).astype(dtype)
    d = (r - np.round(r)).astype(dtype)
    return (dtype(cfg.C) * np.exp(-(d * d) / (dtype(2.0) * sig * sig))).astype(dtype)


# ---------------------------------------------------------------- stencils --
def grad(f: np.ndarray, dx: float):
    """Central gradient, periodic (NS_solver.py:243-247)."""
    dt_ = f.dtype.type
    h = dt_(2 * dx)
    gx = (np.roll(f, -1, axis=0) - np.roll(f, 1, axis=0)) / h
    gy = (np.roll(f, -1, axis=1) - np.roll(f, 1, axis=1)) / h
    return gx.astype(f.dtype), gy.astype(f.dtype)


def laplacian(f: np.ndarray, dx: float) -> np.ndarray:
    """5-point Laplacian, periodic (NS_solver.py:249-255)."""
    dt_ = f.dtype.type
    left = np.roll(f, 1, axis=0)
    right = np.roll(f, -1, axis=0)
    up = np.roll(f, -1, axis=1)
    down = np.roll(f, 1, axis=1)
    return ((left + right + up + down - dt_(4) * f) / dt_(dx ** 2)).astype(f.dtype)


def divergence(u: np.ndarray, dx: float) -> np.ndarray:
    """Central divergence of a (2,N,N) field (NS_solver.py:206-210)."""
    gx, _ = grad(u[0], dx)
    _, gy = grad(u[1], dx)
    return (gx + gy).astype(u.dtype)


def upwind_advect(f: np.ndarray, ux: np.ndarray, uy: np.ndarray, dx: float) -> np.ndarray:
    """First-order upwind -(u.grad)f (NS_solver.py:257-265)."""
    dt_ = f.dtype.type
    h = dt_(dx)
    f_left = np.roll(f, 1, axis=0)
    f_right = np.roll(f, -1, axis=0)
    dfx = np.where(ux >= 0, f - f_left, f_right - f) / h
    f_down = np.roll(f, 1, axis=1)
    f_up = np.roll(f, -1, axis=1)
    dfy = np.where(uy >= 0, f - f_down, f_up - f) / h
    return (-(ux * dfx + uy * dfy)).astype(f.dtype)


def central_advect(f: np.ndarray, ux: np.ndarray, uy: np.ndarray, dx: float) -> np.ndarray:
    """Central -(u.grad)f via the central gradient (NS_solver.py:474-477)."""
    fx, fy = grad(f, dx)
    return (-(ux * fx + uy * fy)).astype(f.dtype)


def advect(f, ux, uy, dx, scheme: str):
    """Advection strategy dispatch (NS_solver.py:491-497)."""
    if scheme == "central":
        return central_advect(f, ux, uy, dx)
    if scheme == "upwind":
        return upwind_advect(f, ux, uy, dx)
    raise ValueError(f"Unknown advection scheme: '{scheme}'. Choose 'central' or 'upwind'.")


# ----------------------------------------------------------------- Poisson --
_FFT_WORKERS = None


def set_fft_workers(n):
    """Run the oracle's FFTs with scipy.fft on n threads (None: numpy.fft).
    Both keep complex64 for float32 input; used by the timed CPU baseline."""
    global _FFT_WORKERS
    _FFT_WORKERS = n


def _fft2(x):
    if _FFT_WORKERS:
        import scipy.fft
        return scipy.fft.fft2(x, workers=_FFT_WORKERS)
    return np.fft.fft2(x)


def _ifft2(x):
    if _FFT_WORKERS:
        import scipy.fft
        return scipy.fft.ifft2(x, workers=_FFT_WORKERS)
    return np.fft.ifft2(x)


def poisson_solve(rhs: np.ndarray, dx: float, inv_k2: np.ndarray | None = None) -> np.ndarray:
    """p = Re ifft2(-fft2(rhs) * inv_k2) with p_hat[0,0] = 0 (NS_solver.py:523-527).

    Solves lap(p) = rhs with the continuous |k|^2.  float32 input runs
    complex64 C2C transforms, float64 input complex128.
    """
    N = rhs.shape[0]
    if inv_k2 is None:
        inv_k2 = poisson_inv_k2(N, dx, rhs.dtype.type)
    ctype = np.complex64 if rhs.dtype == np.float32 else np.complex128
    F = _fft2(rhs.astype(ctype))
    p_hat = (-F * inv_k2).astype(ctype)
    p_hat[0, 0] = 0.0
    return _ifft2(p_hat).real.astype(rhs.dtype)


# ---------------------------------------------------------- time stepping --
def projector_step(u: np.ndarray, f: np.ndarray, cfg: OracleConfig, nu=None,
                   inv_k2: np.ndarray | None = None) -> np.ndarray:
    """One Chorin step (NS_solver.py:671-697):
    u* = u + dt(nu lap u + adv(u) + f);  p = poisson(div(u*)/dt);  u+ = u* - dt grad p.
    """
    dtp = u.dtype.type
    dx = cfg.dx
    dt = dtp(cfg.dt)
    nu = dtp(cfg.nu if nu is None else nu)
    ux, uy = u[0], u[1]
    lap0, lap1 = laplacian(ux, dx), laplacian(uy, dx)
    adv0 = advect(ux, ux, uy, dx, cfg.scheme)
    adv1 = advect(uy, ux, uy, dx, cfg.scheme)
    ux_star = ux + dt * (nu * lap0 + adv0 + f[0])
    uy_star = uy + dt * (nu * lap1 + adv1 + f[1])
    u_star = np.stack([ux_star, uy_star]).astype(u.dtype)
    div_star = divergence(u_star, dx)
    p = poisson_solve((div_star / dt).astype(u.dtype), dx, inv_k2)
    px, py = grad(p, dx)
    return np.stack([ux_star - dt * px, uy_star - dt * py]).astype(u.dtype)


def _split_theta(theta, cfg: OracleConfig, dtype):
    th = np.asarray(theta, dtype=dtype).ravel()
    if th.size not in (2, 3):
        raise ValueError(f"theta must have 2 or 3 entries, got {th.size}")
    nu = th[2] if th.size == 3 else dtype(cfg.nu)
    return th[:2], nu


def full_forcing(theta, t, cfg: OracleConfig, dtype=np.float32) -> np.ndarray:
    """(2,N,N) forcing field, fy = 0 (NS_solver.py:637-640)."""
    fx = forcing_fx(theta, t, cfg, dtype)
    f0 = np.broadcast_to(fx[:, None], (cfg.N, cfg.N)).astype(dtype)
    return np.stack([f0, np.zeros_like(f0)])


def solver_step(u, theta, t, cfg: OracleConfig):
    """SingleCoreNSSolver.step (NS_solver.py:727-730)."""
    dtype = u.dtype.type
    th, nu = _split_theta(theta, cfg, dtype)
    return projector_step(u, full_forcing(th, t, cfg, dtype), cfg, nu=nu)


def rollout(u0: np.ndarray, theta, cfg: OracleConfig, steps: int | None = None,
            return_history: bool = False):
    """SingleCoreNSSolver.rollout (NS_solver.py:732-750).

    ``t = i*dt`` in the array dtype; the objective increment
    ``dt * sum(u*f) * dx**2`` uses the state *before* the step.
    Returns ``(J, u_final)`` (and the list of states if asked).
    """
    dtype = u0.dtype.type
    th, nu = _split_theta(theta, cfg, dtype)
    steps = cfg.steps if steps is None else steps
    inv_k2 = poisson_inv_k2(cfg.N, cfg.dx, dtype)
    dt = dtype(cfg.dt)
    dx2 = dtype(cfg.dx ** 2)
    u = u0.copy()
    J = dtype(0.0)
    hist = [u.copy()] if return_history else None
    for i in range(steps):
        t = dtype(dtype(i) * dt)
        f = full_forcing(th, t, cfg, dtype)
        J = dtype(J + dt * np.sum(u * f, dtype=dtype) * dx2)
        u = projector_step(u, f, cfg, nu=nu, inv_k2=inv_k2)
        if return_history:
            hist.append(u.copy())
    if return_history:
        return J, u, hist
    return J, u


def objective(theta, cfg: OracleConfig, dtype=np.float32):
    """J(theta) from a zero initial condition (NS_solver.py:752-756)."""
    u0 = np.zeros((2, cfg.N, cfg.N), dtype=dtype)
    return rollout(u0, theta, cfg)[0]


def fd_gradient(fn, theta, rel_step: float = 1e-3):
    """Central finite differences with per-parameter step h_i = rel_step*|theta_i|
    (the method of studies.py:306-318 with a relative step)."""
    th = np.asarray(theta, dtype=np.float64)
    g = np.zeros_like(th)
    for i in range(th.size):
        h = rel_step * max(abs(th[i]), 1e-12)
        tp, tm = th.copy(), th.copy()
        tp[i] += h
        tm[i] -= h
        g[i] = (float(fn(tp)) - float(fn(tm))) / (2 * h)
    return g


def rel_l2(a, b) -> float:
    """||a-b|| / (||a|| + 1e-12), the metric of NS_solver.py:912."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / (np.linalg.norm(a) + 1e-12))
