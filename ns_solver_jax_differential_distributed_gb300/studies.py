"""The reference's research studies (studies.py) on the GB300 solver, with
their result formats: ``ViscosityStudy`` (studies.py:51-167),
``GradientBenchmark`` (:271-521), ``SchemeComparisonStudy`` (:526-858) and
``ParameterOptimizationStudy`` (:864-964, in ``optimization.py``).  Each runs
the same simulations as the reference through this package's solver and
writes the same ``.npz`` keys; the plotting methods of the reference are not
provided (no plotting dependency).  Metrics (kinetic energy, vorticity,
velocity statistics) are evaluated on the device.
"""
from __future__ import annotations

import logging
import time
from typing import Callable, Optional, Tuple

import numpy as np
import torch

from .optimization import ParameterOptimizationStudy  # noqa: F401  (re-export)
from .solver import (CONFIG, GaussianForcingField, Grid, Phys, SimConfig, SingleCoreNSSolver, Time,
                     make_grid)

logger = logging.getLogger(__name__)


def _nu_config(config: SimConfig, nu: float, theta, scheme: str) -> SimConfig:
    return SimConfig(N=config.N, L=config.L, nu=float(nu), mu0=config.mu0, sigma0=config.sigma0,
                     C_force=config.C_force, cfl=config.cfl, v_max=config.v_max, t=config.t,
                     theta0=theta, advection_scheme=scheme, obj_tol=config.obj_tol)


def _solver(cfg: SimConfig, scheme: str) -> Tuple[SingleCoreNSSolver, Grid, Phys, Time]:
    grid = make_grid(cfg.N, cfg.L)
    phys = Phys(nu=cfg.nu, mu0=cfg.mu0, sigma0=cfg.sigma0, C=cfg.C_force)
    time_obj = Time(dt=cfg.dt, steps=cfg.steps)
    return SingleCoreNSSolver(grid, phys, time_obj, advection_scheme=scheme), grid, phys, time_obj


def _theta(theta) -> torch.Tensor:
    return torch.as_tensor(np.asarray(theta, np.float32))


# ==========================
# 1. Viscosity Regime Study
# ==========================
class ViscosityStudy:
    """Rollouts from the zero state across viscosities (studies.py:51-167)."""

    def __init__(self, viscosities=None, grid: Optional[Grid] = None, phys_template: Optional[Phys] = None,
                 time_template: Optional[Time] = None, theta=None, config: Optional[SimConfig] = None):
        self.viscosities = (np.array([0.001, 0.005, 0.01, 0.05, 0.1], np.float32) if viscosities is None
                            else np.asarray(viscosities))
        self.grid = grid if grid is not None else make_grid(128, 1.0)
        self.phys_template = phys_template
        self.time_template = time_template
        self.theta = theta if theta is not None else np.array([1.0, 0.5], np.float32)
        self.config = config if config is not None else CONFIG
        self.results: dict = {}
        logger.info(f"ViscosityStudy initialized with {len(self.viscosities)} viscosity values")

    def _compute_kinetic_energy(self, u: torch.Tensor) -> float:
        return float(0.5 * torch.sum(u[0] ** 2 + u[1] ** 2) * (self.grid.dx ** 2))

    def _compute_vorticity(self, u: torch.Tensor, dx: float) -> torch.Tensor:
        """omega = d(u_y)/dx - d(u_x)/dy, central differences (studies.py:79-92)."""
        duy_dx = (torch.roll(u[1], -1, 0) - torch.roll(u[1], 1, 0)) / (2 * dx)
        dux_dy = (torch.roll(u[0], -1, 1) - torch.roll(u[0], 1, 1)) / (2 * dx)
        return duy_dx - dux_dy

    def _compute_velocity_stats(self, u: torch.Tensor) -> dict:
        speed = torch.sqrt(u[0] ** 2 + u[1] ** 2)
        return {"speed_max": float(speed.max()), "speed_mean": float(speed.mean()),
                "speed_std": float(speed.std(unbiased=False)), "ux_max": float(u[0].abs().max()),
                "uy_max": float(u[1].abs().max())}

    def run_sweep(self) -> dict:
        results = {}
        for nu in self.viscosities:
            logger.info(f"Running simulation for nu={float(nu):.4f}")
            cfg = _nu_config(self.config, float(nu), self.theta, self.config.advection_scheme)
            solver, grid, _, _ = _solver(cfg, cfg.advection_scheme)
            u0 = torch.zeros((2, cfg.N, cfg.N), dtype=torch.float32, device=solver.device)
            J, u_final = solver.rollout(u0, _theta(self.theta).to(solver.device))
            ke = self._compute_kinetic_energy(u_final)
            results[float(nu)] = {"dt": cfg.dt, "objective": float(J), "kinetic_energy": ke,
                                  "velocity_stats": self._compute_velocity_stats(u_final),
                                  "vorticity": self._compute_vorticity(u_final, grid.dx), "u_final": u_final}
            logger.info(f"dt={cfg.dt:.6e}, obj={float(J):.6e}, KE={ke:.6e}")
        self.results = results
        return results

    def save_results(self, filename: str = "result/viscosity_study_results.npz") -> None:
        """studies.py:154-167."""
        if not self.results:
            logger.warning("No results to save")
            return
        data = {}
        for nu, r in self.results.items():
            data[f"nu_{nu:.4f}_objective"] = r["objective"]
            data[f"nu_{nu:.4f}_kinetic_energy"] = r["kinetic_energy"]
            data[f"nu_{nu:.4f}_dt"] = r["dt"]
        np.savez(filename, **data)
        logger.info(f"Saved results to {filename}")


# ==========================
# 2. Gradient Research
# ==========================
class GradientBenchmark:
    """Adjoint gradient against central finite differences over a sweep of
    step sizes, with the gradient's timing (studies.py:271-521).  The
    reference's "JAX" fields hold this package's discrete-adjoint gradient:
    ``time_jax_compile_first`` is the first call (plan and workspace set-up),
    ``time_jax_exec_mean/std`` the steady state."""

    def __init__(self, objective: Callable, grad_jax: Callable, param_vectors: Optional[list] = None,
                 epsilon_range=None, jax_timing_runs: int = 5, config: Optional[SimConfig] = None):
        self.objective = objective
        self.grad_jax = grad_jax
        self.config = config or CONFIG
        self.param_vectors = param_vectors or [np.array([1.0, 0.5], np.float32), np.array([0.5, 1.0], np.float32),
                                               np.array([2.0, 0.2], np.float32)]
        self.epsilon_range = (np.logspace(-7, -1, 20).astype(np.float32) if epsilon_range is None
                              else np.asarray(epsilon_range))
        self.jax_timing_runs = max(1, int(jax_timing_runs))
        self.results: dict = {}

    @staticmethod
    def _sync():
        if torch.cuda.is_available():
            torch.cuda.synchronize()

    def _compute_fd_gradient(self, theta: np.ndarray, epsilon: float) -> np.ndarray:
        g = np.zeros(len(theta), np.float32)
        for i in range(len(theta)):
            tp, tm = np.array(theta, np.float32), np.array(theta, np.float32)
            tp[i] += np.float32(epsilon)
            tm[i] -= np.float32(epsilon)
            g[i] = (float(self.objective(tp)) - float(self.objective(tm))) / (2 * epsilon)
        return g

    def sweep_epsilon(self, theta) -> dict:
        theta = np.asarray(theta, np.float32)
        t0 = time.perf_counter()
        g = self.grad_jax(theta)
        self._sync()
        t_first = time.perf_counter() - t0
        samples = []
        for _ in range(self.jax_timing_runs):
            t1 = time.perf_counter()
            g = self.grad_jax(theta)
            self._sync()
            samples.append(time.perf_counter() - t1)
        g = np.asarray(torch.as_tensor(g).detach().cpu(), np.float32)
        sweep = {}
        for eps in self.epsilon_range:
            t0 = time.time()
            fd = self._compute_fd_gradient(theta, float(eps))
            t_fd = time.time() - t0
            abs_err = float(np.linalg.norm(g - fd))
            sweep[float(eps)] = {"grad_fd": fd, "abs_error": abs_err,
                                 "rel_error": abs_err / (float(np.linalg.norm(fd)) + 1e-12), "time_fd": t_fd}
        mean = float(np.mean(samples))
        return {"grad_jax": g, "time_jax": mean, "time_jax_compile_first": t_first, "time_jax_exec_mean": mean,
                "time_jax_exec_std": float(np.std(samples)), "epsilon_sweep": sweep}

    def run_all(self) -> dict:
        self.results = {idx: self.sweep_epsilon(th) for idx, th in enumerate(self.param_vectors)}
        return self.results

    def save_results(self, filename: str = "result/gradient_benchmark_results.npz") -> None:
        """studies.py:502-521."""
        if not self.results:
            logger.warning("No results to save")
            return
        data = {}
        for idx, r in self.results.items():
            for k in ("time_jax", "time_jax_compile_first", "time_jax_exec_mean", "time_jax_exec_std"):
                data[f"param_{idx}_{k}"] = r[k]
            eps = sorted(r["epsilon_sweep"])
            data[f"param_{idx}_epsilons"] = np.array(eps)
            data[f"param_{idx}_rel_errors"] = np.array([r["epsilon_sweep"][e]["rel_error"] for e in eps])
            data[f"param_{idx}_abs_errors"] = np.array([r["epsilon_sweep"][e]["abs_error"] for e in eps])
            data[f"param_{idx}_times_fd"] = np.array([r["epsilon_sweep"][e]["time_fd"] for e in eps])
        np.savez(filename, **data)
        logger.info(f"Saved to {filename}")


# ==========================
# 3. Upwind/central scheme comparison
# ==========================
class SchemeComparisonStudy:
    """Central against upwind advection across viscosities, with the
    per-step objective and maximum speed (studies.py:526-858).  The history
    is accumulated on the device and read back once per run."""

    def __init__(self, viscosities=None, grid: Optional[Grid] = None, config: Optional[SimConfig] = None):
        self.viscosities = (np.array([0.005, 0.01, 0.05], np.float32) if viscosities is None
                            else np.asarray(viscosities))
        self.schemes = ["central", "upwind"]
        self.grid = grid or make_grid(128, 1.0)
        self.config = config or CONFIG
        self.results: dict = {}

    def run_comparison(self, theta, make_solver_fn: Optional[Callable] = None) -> dict:
        results = {}
        for scheme in self.schemes:
            sr = {}
            for nu in self.viscosities:
                cfg = _nu_config(self.config, float(nu), theta, scheme)
                solver, grid, phys, time_obj = _solver(cfg, scheme)
                u0 = torch.zeros((2, cfg.N, cfg.N), dtype=torch.float32, device=solver.device)
                J, u_final, hist = self._rollout_with_history(solver, u0, theta, grid, phys, time_obj)
                speed = torch.sqrt(u_final[0] ** 2 + u_final[1] ** 2)
                ke = float(0.5 * torch.sum(u_final[0] ** 2 + u_final[1] ** 2) * (grid.dx ** 2))
                sr[float(nu)] = {"objective": float(J), "kinetic_energy": ke, "max_velocity": float(speed.max()),
                                 "convergence_history": hist, "u_final": u_final, "dt": cfg.dt}
            results[scheme] = sr
        self.results = results
        return results

    def _rollout_with_history(self, solver: SingleCoreNSSolver, u0: torch.Tensor, theta, grid: Grid, phys: Phys,
                              time_obj: Time):
        """Step by step with the J of studies.py:623-640: the objective and
        the maximum speed of the state before each step."""
        dev = solver.device
        th = _theta(theta).to(dev)
        forcing = GaussianForcingField(grid, phys)
        steps = time_obj.steps
        Js = torch.empty(steps, dtype=torch.float32, device=dev)
        vmax = torch.empty(steps, dtype=torch.float32, device=dev)
        J = torch.zeros((), dtype=torch.float32, device=dev)
        u = u0
        for i in range(steps):
            t = i * time_obj.dt
            f = forcing(th, t)
            J = J + time_obj.dt * torch.sum(u * f) * (grid.dx ** 2)
            Js[i] = J
            vmax[i] = torch.sqrt(u[0] ** 2 + u[1] ** 2).max()
            u = solver.step(u, th, t)
        Jh, vh = Js.cpu().numpy(), vmax.cpu().numpy()
        hist = [{"step": i, "objective": float(Jh[i]), "time": float(i * time_obj.dt),
                 "max_velocity": float(vh[i])} for i in range(steps)]
        return J, u, hist

    def save_results(self, filename: str = "result/scheme_comparison_results.npz") -> None:
        """studies.py:839-858."""
        if not self.results:
            logger.warning("No results to save")
            return
        data = {}
        for scheme, sr in self.results.items():
            for nu, r in sr.items():
                for k in ("objective", "kinetic_energy", "max_velocity", "dt"):
                    data[f"{scheme}_nu_{nu:.4f}_{k}"] = r[k]
        np.savez(filename, **data)
        logger.info(f"Saved results to {filename}")
