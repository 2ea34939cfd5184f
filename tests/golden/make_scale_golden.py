"""Oracle fixtures for the two large parity cases (run on a CPU host; slow).

The large cases cannot run through the oracle inside a GPU test in reasonable
time, so this script runs them once and stores compact, size-independent
summaries under tests/golden/:

* ``scale_N4096_<scheme>.npz`` -- the headline rollout (N=4096 on [0, 2 pi]^2,
  200 steps, dt=2.5e-4, nu=1e-4, seeded spectral u0 with |k| <= 32, seeded
  theta; the reference's rollout, NS_solver.py:732-750) through the float32
  oracle and the float64 oracle: both objectives J, every row's L2 norm of
  both velocity components, a sample of full rows of u_final (rows 17 + 256 m,
  m = 0..15, stored as float32), and the full-field rel-L2 between the float32
  and float64 oracles (the metric of NS_solver.py:912).
* ``grad_N1024_upwind.json`` -- the differentiation case (N=1024, 1000 steps,
  dt=1e-3, nu=5e-4, upwind): J in float32 and float64 and the central finite-
  difference gradient of the float64 oracle's J with respect to [A, B, nu]
  with relative steps 1e-3 and 5e-4 per parameter (the method of
  studies.py:306-318; the two steps bound the truncation error), and for A
  also with relative steps 1e-5 and 1e-7.  The forcing's period-1 wrap
  d = (x - mu) - round(x - mu) (NS_solver.py:626) gives f_x a kink in mu at
  every row and step; at this size thousands of them fall within +-1e-3 A,
  so wide steps average the slope over kinks, while reverse-mode
  differentiation (jax.grad, the discrete adjoint) returns the derivative at
  the point, which the small steps resolve (1e-7 A sits between the kink
  spacing and float64 noise).

Each rollout runs in its own process of a spawn-started pool (the oracle's
array code is single-threaded), one process per core by default.

Usage:  python tests/golden/make_scale_golden.py [--only scale|grad] [--workers K]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ns_oracle as O  # noqa: E402
from ns_solver_jax_differential_distributed_gb300.workloads import (  # noqa: E402
    GRAD_N1024, PLAIN_SCALE_CENTRAL, PLAIN_SCALE_UPWIND)

SAMPLE_ROWS = 17 + 256 * np.arange(16)
# (relative step, parameters) of the finite differences of the gradient case
FD_STEPS = ((1e-3, (0, 1, 2)), (5e-4, (0, 1)), (1e-5, (0,)), (1e-7, (0,)))


def _cfg(w):
    return O.OracleConfig(N=w.N, L=w.L, nu=w.nu, dt=w.dt, steps=w.steps, scheme=w.scheme)


WORKLOADS = {w.name: w for w in (PLAIN_SCALE_CENTRAL, PLAIN_SCALE_UPWIND, GRAD_N1024)}


def _job(args):
    """One oracle rollout in a worker process: (workload, dtype, theta) ->
    (J, u_final or None, seconds)."""
    name, dtype, theta, keep_u = args
    O.set_fft_workers(1)
    w = WORKLOADS[name]
    dt = np.float32 if dtype == "f32" else np.float64
    t0 = time.perf_counter()
    J, u = O.rollout(w.u0().astype(dt), np.asarray(theta, dtype=dt), _cfg(w))
    return float(J), (u if keep_u else None), time.perf_counter() - t0


def scale_summary(w, r32, r64):
    (J32, u32, t32), (J64, u64, t64) = r32, r64
    out = {
        "J32": np.float64(J32), "J64": np.float64(J64),
        "rownorm32": np.sqrt(np.sum(u32.astype(np.float64) ** 2, axis=2)),
        "rownorm64": np.sqrt(np.sum(u64 ** 2, axis=2)),
        "rows": SAMPLE_ROWS.astype(np.int32),
        "u32_rows": u32[:, SAMPLE_ROWS, :].astype(np.float32),
        "u64_rows": u64[:, SAMPLE_ROWS, :].astype(np.float32),
        "rel_l2_32_vs_64_full": np.float64(O.rel_l2(u64, u32)),
        "rel_l2_32_vs_64_rows": np.float64(O.rel_l2(u64[:, SAMPLE_ROWS, :], u32[:, SAMPLE_ROWS, :])),
        "seconds_32_64": np.array([t32, t64]),
    }
    path = os.path.join(HERE, f"scale_N{w.N}_{w.scheme}.npz")
    np.savez_compressed(path, **out)
    print(f"{w.name}: J32={J32:.9g} J64={J64:.9g} rel32v64={out['rel_l2_32_vs_64_full']:.3e} "
          f"({t32:.0f} s, {t64:.0f} s) -> {path}", flush=True)


def grad_jobs(w):
    th = w.theta().astype(np.float64)
    jobs = [(w.name, "f32", th.tolist(), False), (w.name, "f64", th.tolist(), False)]
    keys = [("J32",), ("J64",)]
    for rs, params in FD_STEPS:
        for i in params:
            h = rs * abs(th[i])
            for sgn in (1, -1):
                t = th.copy()
                t[i] += sgn * h
                jobs.append((w.name, "f64", t.tolist(), False))
                keys.append(("fd", rs, i, sgn, h))
    return jobs, keys


def grad_summary(w, keys, results):
    th = w.theta().astype(np.float64)
    vals = {}
    secs = 0.0
    for k, (J, _, s) in zip(keys, results):
        vals[k] = J
        secs += s
    fd = {}
    for rs, params in FD_STEPS:
        g = []
        for i in params:
            kp = [k for k in keys if k[0] == "fd" and k[1] == rs and k[2] == i and k[3] == 1][0]
            km = [k for k in keys if k[0] == "fd" and k[1] == rs and k[2] == i and k[3] == -1][0]
            g.append((vals[kp] - vals[km]) / (2 * kp[4]))
        fd[str(rs)] = g
    out = {"workload": w.name, "N": w.N, "steps": w.steps, "dt": w.dt, "nu": w.nu, "scheme": w.scheme,
           "theta": [float(x) for x in w.theta()], "J32": vals[("J32",)], "J64": vals[("J64",)],
           "fd64": fd, "cpu_seconds": secs,
           "generator": {"numpy": np.__version__, "machine": platform.machine()}}
    path = os.path.join(HERE, f"grad_N{w.N}_{w.scheme}.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(f"{w.name}: J64={out['J64']:.12g} fd={fd} -> {path}", flush=True)


def main():
    import multiprocessing as mp
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["scale", "grad"], default=None)
    ap.add_argument("--workers", type=int, default=len(os.sched_getaffinity(0)))
    args = ap.parse_args()
    jobs, tags = [], []
    if args.only in (None, "scale"):
        for w in (PLAIN_SCALE_CENTRAL, PLAIN_SCALE_UPWIND):
            th = w.theta().astype(np.float64).tolist()
            jobs += [(w.name, "f64", th, True), (w.name, "f32", th, True)]
            tags += [("scale", w.name, "f64"), ("scale", w.name, "f32")]
    gkeys = []
    if args.only in (None, "grad"):
        gj, gkeys = grad_jobs(GRAD_N1024)
        jobs += gj
        tags += [("grad",)] * len(gj)
    with mp.get_context("spawn").Pool(args.workers) as pool:
        results = pool.map(_job, jobs, chunksize=1)
    by = dict(zip(tags, results)) if args.only != "grad" else {}
    for w in (PLAIN_SCALE_CENTRAL, PLAIN_SCALE_UPWIND):
        if ("scale", w.name, "f32") in by:
            scale_summary(w, by[("scale", w.name, "f32")], by[("scale", w.name, "f64")])
    if gkeys:
        gres = [r for t, r in zip(tags, results) if t == ("grad",)]
        grad_summary(GRAD_N1024, gkeys, gres)


if __name__ == "__main__":
    main()
