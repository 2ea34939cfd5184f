"""Extract golden vectors from the reference's shipped result artefacts.

The reference (helmhlotz/ns_solver_jax_differential_distributed) ships the
outputs of its own runs under ``result/``.  JAX is not installed here, so these
artefacts are the reference's own outputs that pin the CPU oracle.  This script
reads them from a reference checkout and writes small fixtures next to itself:

* ``reference_results.json`` -- objectives / kinetic energies / max speeds of the
  viscosity and scheme studies (studies.py:118-167, 552-601), the SGD(lr=0.1)
  trajectory of the optimisation study (studies.py:890-934), from which the JAX
  reverse-mode gradient follows as (theta_k - theta_{k+1}) / 0.1, the
  trajectories of all four optimisers of that study, the finite-difference
  error sweep of the gradient benchmark (studies.py:271-521), and the
  configurations each number was produced with;
* ``speed_single_N128.npy`` -- |u| after runner.py's single-device run at
  N=128 (runner.py:115-175, sample_config/config_N_128.json);
* ``speed_P8_N512_sub4.npy`` -- every 4th point (both axes) of |u| after the
  N=512 run (sample_config/config_N_512.json), plus its full-field norm in
  the JSON.

Usage:  python tests/golden/make_golden.py /path/to/reference
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def simconfig_dt(N: int, L: float, nu: float, cfl: float = 0.4, v_max: float = 1.0) -> float:
    """SimConfig.dt (NS_solver.py:75-79): min of CFL and diffusive limits, rounded
    through float32 by jnp.minimum."""
    dx = L / N
    return float(np.float32(min(cfl * dx / v_max, dx * dx / (4.0 * nu))))


def simconfig_steps(t: float, dt: float) -> int:
    """SimConfig.steps (NS_solver.py:67-68)."""
    return int(math.ceil(t / dt))


def main(ref: str) -> None:
    res = os.path.join(ref, "result")
    out: dict = {"source": "reference result/ artefacts", "studies": {}}

    # Defaults of the studies: SimConfig() with N=128, L=1, t=0.5, theta=[1, 0.5].
    base = dict(N=128, L=1.0, t=0.5, theta=[1.0, 0.5])

    visc = np.load(os.path.join(res, "viscosity_study_results.npz"))
    rows = []
    for nu in (0.001, 0.005, 0.01, 0.05, 0.1):
        dt = simconfig_dt(128, 1.0, nu)
        rows.append(dict(base, nu=nu, scheme="central", dt=dt, steps=simconfig_steps(0.5, dt),
                         objective=float(visc[f"nu_{nu:.4f}_objective"]),
                         kinetic_energy=float(visc[f"nu_{nu:.4f}_kinetic_energy"]),
                         dt_saved=float(visc[f"nu_{nu:.4f}_dt"])))
    out["studies"]["viscosity"] = rows

    sch = np.load(os.path.join(res, "scheme_comparison_results.npz"))
    rows = []
    for scheme in ("central", "upwind"):
        for nu in (0.005, 0.01, 0.05):
            dt = simconfig_dt(128, 1.0, nu)
            key = f"{scheme}_nu_{nu:.4f}"
            rows.append(dict(base, nu=nu, scheme=scheme, dt=dt, steps=simconfig_steps(0.5, dt),
                             objective=float(sch[key + "_objective"]),
                             kinetic_energy=float(sch[key + "_kinetic_energy"]),
                             max_velocity=float(sch[key + "_max_velocity"]),
                             dt_saved=float(sch[key + "_dt"])))
    out["studies"]["scheme"] = rows

    opt = np.load(os.path.join(res, "optimization_study_results.npz"))
    dt = simconfig_dt(128, 1.0, 0.01)
    out["studies"]["sgd"] = dict(
        base, nu=0.01, scheme="central", dt=dt, steps=simconfig_steps(0.5, dt), lr=0.1,
        parameters=opt["SGD (lr=0.1)_parameters"].astype(np.float64).tolist(),
        objectives=opt["SGD (lr=0.1)_objectives"].astype(np.float64).tolist())
    # All four optimiser trajectories of ParameterOptimizationStudy
    # (studies.py:879-884, optax 0.2.4 defaults), 100 steps from theta0.
    runs = []
    for name in ("Adam (lr=0.01)", "Adam (lr=0.001)", "SGD (lr=0.1)", "RMSprop (lr=0.01)"):
        runs.append(dict(name=name, obj_initial=float(opt[f"{name}_obj_initial"]),
                         obj_final=float(opt[f"{name}_obj_final"]),
                         improvement=float(opt[f"{name}_improvement"]),
                         parameters=opt[f"{name}_parameters"].astype(np.float64).tolist(),
                         objectives=opt[f"{name}_objectives"].astype(np.float64).tolist()))
    out["studies"]["optimizers"] = dict(base, nu=0.01, scheme="central", dt=dt,
                                        steps=simconfig_steps(0.5, dt), optim_steps=100, runs=runs)

    # GradientBenchmark (studies.py:271-521): central-FD vs JAX gradient over
    # 20 step sizes for three parameter vectors, config of the optimiser study.
    gb = np.load(os.path.join(res, "gradient_benchmark_results.npz"))
    out["studies"]["gradient_benchmark"] = dict(
        base, nu=0.01, scheme="central", dt=dt, steps=simconfig_steps(0.5, dt),
        param_vectors=[[1.0, 0.5], [0.5, 0.5], [2.0, 1.0]],  # studies.py:1064-1074
        epsilons=gb["param_0_epsilons"].astype(np.float64).tolist(),
        rel_errors=[gb[f"param_{i}_rel_errors"].astype(np.float64).tolist() for i in range(3)],
        time_jax_exec_mean=[float(gb[f"param_{i}_time_jax_exec_mean"]) for i in range(3)])

    # Speed fields of runner.py (sample configs: nu=1e-4, t=0.5, central, L=1).
    s128 = np.load(os.path.join(res, "velocity_magnitude_single_N128.npy")).astype(np.float32)
    np.save(os.path.join(HERE, "speed_single_N128.npy"), s128)
    s512 = np.load(os.path.join(res, "velocity_magnitude_distributed_P8_N512.npy")).astype(np.float32)
    np.save(os.path.join(HERE, "speed_P8_N512_sub4.npy"), np.ascontiguousarray(s512[::4, ::4]))
    fields = []
    for N, name in ((128, "speed_single_N128.npy"), (512, "speed_P8_N512_sub4.npy")):
        dt = simconfig_dt(N, 1.0, 1e-4)
        full = s128 if N == 128 else s512
        fields.append(dict(N=N, L=1.0, nu=1e-4, t=0.5, theta=[1.0, 0.5], scheme="central",
                           dt=dt, steps=simconfig_steps(0.5, dt), file=name,
                           stride=1 if N == 128 else 4,
                           full_norm=float(np.linalg.norm(full.astype(np.float64))),
                           full_mean=float(full.astype(np.float64).mean())))
    out["speed_fields"] = fields

    with open(os.path.join(HERE, "reference_results.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", os.path.join(HERE, "reference_results.json"))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
