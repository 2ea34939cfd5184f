"""Command-line entry point (runner.py of the reference, single-device path).

    python -m ns_solver_jax_differential_distributed_gb300.runner --config sample_config/config_N_128.json

Same flags as the reference's runner (runner.py:31-55): ``--config`` (JSON
config; missing fields fall back to the defaults), ``--profile`` (stage-wise
timing), ``--profile-warmup`` and ``--profile-runs``.  It builds the solver
from the config, runs the rollout from the zero state and writes the speed
field |u| to ``result/velocity_magnitude_single_N{N}.npy`` (the reference's
file name and content, runner.py:162-175).  The reference also draws a PNG
with matplotlib; this package has no plotting dependency and writes the array
only.  The distributed comparison of the reference (jax.device_count() > 1)
is out of scope: one GPU runs the single-device solver, and ``--profile``
times its stages.
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np
import torch

from .solver import Phys, SingleCoreNSSolver, Time, load_config, make_grid, setup_logger

logger = setup_logger(__name__)


def build_parser() -> argparse.ArgumentParser:
    """The reference's CLI parser (runner.py:31-55)."""
    parser = argparse.ArgumentParser(description="Navier-Stokes CFD Solver")
    parser.add_argument("--config", type=str, default=None,
                        help="Path to a JSON config file. Missing fields fall back to defaults.")
    parser.add_argument("--profile", action="store_true",
                        help="Run stage-wise profiling of the single-device solver.")
    parser.add_argument("--profile-warmup", type=int, default=1,
                        help="Number of warmup runs per profiled kernel (excluded from statistics).")
    parser.add_argument("--profile-runs", type=int, default=5, help="Number of measured runs per profiled kernel.")
    return parser


def main(argv=None) -> dict:
    args = build_parser().parse_args(argv)
    logger.info("=" * 80)
    logger.info("NAVIER-STOKES CFD SOLVER (GB300)")
    logger.info("=" * 80)
    config = load_config(args.config)
    grid = make_grid(config.N, L=config.L)
    phys = Phys(nu=config.nu, mu0=config.mu0, sigma0=config.sigma0, C=config.C_force)
    time_cfg = Time(dt=config.dt, steps=config.steps)
    theta = config.theta0
    solver = SingleCoreNSSolver(grid, phys, time_cfg, advection_scheme=config.advection_scheme)
    logger.info(f"Advection scheme: {config.advection_scheme}; N={config.N}, dt={config.dt}, steps={config.steps}")

    if args.profile:
        from .profile_stages import profile_solver_kernels
        profile_solver_kernels(solver, theta, warmup=args.profile_warmup, runs=args.profile_runs, logger=logger)

    u0 = torch.zeros((2, config.N, config.N), dtype=torch.float32, device=solver.device)
    torch.cuda.synchronize(solver.device)
    t0 = time.perf_counter()
    _, u_single = solver.rollout(u0, theta)
    torch.cuda.synchronize(solver.device)
    t_single = time.perf_counter() - t0
    logger.info(f"Total time used for single-core solver: {t_single:.3f}s")

    speed = torch.sqrt(u_single[0] ** 2 + u_single[1] ** 2).cpu().numpy()
    os.makedirs("result", exist_ok=True)
    save_npy = f"result/velocity_magnitude_single_N{config.N}.npy"
    np.save(save_npy, np.array(speed))
    logger.info(f"Saved: {save_npy}")
    logger.info("DONE.")
    return {"path": save_npy, "seconds": t_single}


if __name__ == "__main__":
    main()
