"""Per-stage timing of one solver step (the stage split of the reference's
solver_profiler.py: advection_diffusion -> the fused stencil, pressure_solve ->
the three FFT kernels), and the ``ProfileSummary`` / ``benchmark_callable``
contract of solver_profiler.py:14-61 for host-level timing.

    python -m ns_solver_jax_differential_distributed_gb300.profile_stages --N 4096 --reps 1

runs one warm step and then `reps` launches of each stage kernel with CUDA
events (cold L2 per launch) and prints the mean time, the achieved bandwidth
for the stage's algorithmic bytes and the fraction of the measured HBM peak.
It launches few kernels, so it is the command to capture under ncu.

    python -m ns_solver_jax_differential_distributed_gb300.profile_stages --N 4096 --scheme upwind --adjoint 6

times the backward steps of a 6-step gradient (adjoint stencil and FFT passes
per step, every state stored) instead; ``--fused -1`` times the two kernels of
the fused-row step (nsgb_plan_set_fused) instead of the four.

    python -m ns_solver_jax_differential_distributed_gb300.profile_stages --N 128 --grad-batch 4

runs COUNT gradient solves of N (12 steps, checkpoints every 4, seeded u0 and
theta per solve) as one gradient batch (nsgb_grad_batch_advance) after a
warm-up batch, and prints the batch's device time beside the solves run one
after another: the command whose launch list shows the batched kernels.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time
from dataclasses import dataclass
from typing import Callable, List

import numpy as np


@dataclass(frozen=True)
class ProfileSummary:
    """solver_profiler.py:14-20."""
    label: str
    mean_sec: float
    min_sec: float
    max_sec: float
    std_sec: float


def benchmark_callable(label: str, fn: Callable, *args, warmup: int = 1, runs: int = 5) -> ProfileSummary:
    """Warm-up calls, then `runs` timed calls with a device synchronisation
    after each (solver_profiler.py:36-61)."""
    import torch

    def block(x):
        if torch.cuda.is_available():
            torch.cuda.synchronize()
        return x

    for _ in range(max(0, warmup)):
        block(fn(*args))
    samples: List[float] = []
    for _ in range(max(1, runs)):
        t0 = time.perf_counter()
        block(fn(*args))
        samples.append(time.perf_counter() - t0)
    a = np.array(samples, dtype=np.float64)
    return ProfileSummary(label, float(a.mean()), float(a.min()), float(a.max()), float(a.std()))


class SolverKernelProfiler:
    """Stage profiling of the single-core solver (solver_profiler.py:23-240,
    whose distributed half is out of scope): forcing, advection_diffusion,
    pressure_solve and projection through the solver's own strategy objects
    (each stage one or a few kernels of libnsgb), then the fused full step and
    the full rollout."""

    def __init__(self, logger=None):
        import logging
        self.logger = logger if logger is not None else logging.getLogger(__name__)

    @classmethod
    def benchmark_callable(cls, label: str, fn: Callable, *args, warmup: int = 1, runs: int = 5) -> ProfileSummary:
        return benchmark_callable(label, fn, *args, warmup=warmup, runs=runs)

    def _log_profile_table(self, title: str, rows: List[ProfileSummary]) -> None:
        self.logger.info("-" * 80)
        self.logger.info(title)
        self.logger.info("-" * 80)
        self.logger.info(f"{'Kernel':36s} {'mean [s]':>12s} {'min [s]':>12s} {'max [s]':>12s} {'std [s]':>12s}")
        for row in rows:
            self.logger.info(f"{row.label:36s} {row.mean_sec:12.6f} {row.min_sec:12.6f} {row.max_sec:12.6f} "
                             f"{row.std_sec:12.6f}")

    def profile_solver_kernels(self, single, theta, warmup: int = 1, runs: int = 5) -> List[ProfileSummary]:
        import torch
        dev = single.device
        N, dt = single.grid.N, single.time.dt
        pr = single.projector
        ops, adv, poi, nu = pr.ops, pr.advection, pr.poisson, pr.nu
        theta = torch.as_tensor(theta, dtype=torch.float32).to(dev)
        u0 = torch.zeros((2, N, N), dtype=torch.float32, device=dev)
        t0 = 0.0

        def s_forcing(th, t):
            return single.forcing(th, t)

        def s_advec_diff(u, f):
            ux, uy = u[0], u[1]
            ux_s = ux + dt * (nu * ops.laplacian(ux) + adv.advect(ux, ux, uy, ops) + f[0])
            uy_s = uy + dt * (nu * ops.laplacian(uy) + adv.advect(uy, ux, uy, ops) + f[1])
            return torch.stack([ux_s, uy_s])

        def s_pressure(us):
            return poi(ops.divergence(us) / dt)

        def s_projection(us, p):
            px, py = ops.grad(p)
            return torch.stack([us[0] - dt * px, us[1] - dt * py])

        f = s_forcing(theta, t0)
        us = s_advec_diff(u0, f)
        p = s_pressure(us)
        rows = [
            self.benchmark_callable("single: forcing", s_forcing, theta, t0, warmup=warmup, runs=runs),
            self.benchmark_callable("single: advection_diffusion", s_advec_diff, u0, f, warmup=warmup, runs=runs),
            self.benchmark_callable("single: pressure_solve", s_pressure, us, warmup=warmup, runs=runs),
            self.benchmark_callable("single: projection", s_projection, us, p, warmup=warmup, runs=runs),
            self.benchmark_callable("single: full_step", single.step, u0, theta, t0, warmup=warmup, runs=runs),
            self.benchmark_callable("single: full_rollout", single.rollout, u0, theta, warmup=warmup,
                                    runs=max(1, min(runs, 3))),
        ]
        self._log_profile_table("Single-core solver stages", rows)
        return rows


def profile_solver_kernels(single_solver, theta, warmup: int = 1, runs: int = 5, logger=None):
    """solver_profiler.py's entry point for the single-core solver."""
    return SolverKernelProfiler(logger).profile_solver_kernels(single_solver, theta, warmup=warmup, runs=runs)


def main(argv=None):
    import torch
    from . import _build, _native
    from .workloads import spectral_u0, theta_draw
    ap = argparse.ArgumentParser()
    ap.add_argument("--N", type=int, default=4096)
    ap.add_argument("--scheme", default="central")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--no-flush", action="store_true")
    ap.add_argument("--tiles", default="", help="tw,th,rows,cols")
    ap.add_argument("--radix", default="", help="FFT radix of the row and column passes: rows,cols")
    ap.add_argument("--adjoint", type=int, default=0, metavar="STEPS",
                    help="instead: time the backward steps of a STEPS-step gradient (every state stored)")
    ap.add_argument("--adjoint-tiles", default="", help="tw,th of the adjoint stencil")
    ap.add_argument("--tuned", action="store_true",
                    help="apply the autotuner's cached shapes for (N, scheme) first (as bench.py runs them)")
    ap.add_argument("--grad-batch", type=int, default=0, metavar="COUNT",
                    help="instead: COUNT gradient solves of N as one batch, against one after another")
    ap.add_argument("--fused", type=int, default=0, metavar="ROWS",
                    help="time the two-kernel step with the fused row kernel (bands of ROWS rows; -1: the "
                         "band that fits every cluster at once)")
    args = ap.parse_args(argv)
    _build.build()
    dev = torch.device("cuda")
    L = 2 * math.pi
    u0 = torch.from_numpy(spectral_u0(args.N, min(32, args.N // 4), 0)).to(dev)
    th = torch.from_numpy(theta_draw(1e-4, 0)).to(dev)
    plan = _native.get_plan(args.N, L, dev)
    if args.tuned:
        from . import autotune
        if not autotune.apply_cached(args.N, L, args.scheme, dev):
            raise SystemExit(f"no cached autotune shapes for N={args.N} {args.scheme}")
    if args.radix:
        plan.set_fft_radix(*[int(x) for x in args.radix.split(",")])
    if args.tiles:
        plan.set_tiles(*[int(x) for x in args.tiles.split(",")])
    if args.adjoint_tiles:
        plan.set_adjoint_tiles(*[int(x) for x in args.adjoint_tiles.split(",")])
    plan.set_fused(args.fused)
    if args.grad_batch:
        from .ensemble import GradientBatch
        steps, every, nu = 12, 4, 1e-3
        dt = 0.4 / args.N
        cases = [(torch.from_numpy(spectral_u0(args.N, min(32, args.N // 4), k)).to(dev),
                  torch.from_numpy(theta_draw(nu, k)).to(dev)) for k in range(args.grad_batch)]

        def batched():
            gb = GradientBatch(dev)
            ids = [gb.add(u, t, steps, every, L, nu, dt, args.scheme) for u, t in cases]
            gb.run(64)
            return [gb.result(k)[1] for k in ids]

        def sequential():
            return [_native.rollout_grad_raw(u, t, steps, every, L, nu, dt, args.scheme, want_u_final=False,
                                             own_workspace=True)[1] for u, t in cases]

        res = {}
        for name, fn in (("batched", batched), ("sequential", sequential)):
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            g = fn()
            e1.record()
            torch.cuda.synchronize()
            res[name] = (e0.elapsed_time(e1), g)
        same = all(torch.equal(a, b) for a, b in zip(res["batched"][1], res["sequential"][1]))
        print(json.dumps({"N": args.N, "scheme": args.scheme, "solves": args.grad_batch, "steps": steps,
                          "every": every, "batched_ms": round(res["batched"][0], 4),
                          "sequential_ms": round(res["sequential"][0], 4), "bitwise_equal": same}))
        return
    if args.adjoint:
        # forward once, then `reps` backward phases (adjoint stencil + FFT
        # passes per step), timed with CUDA events; few launches, so the
        # command to capture the adjoint kernel under ncu
        sess = _native.GradSession(u0, th, args.adjoint, 1, L, 1e-4, 2.5e-4, args.scheme)
        sess.forward()
        for _ in range(2):  # the second identical call captures the graph later calls replay
            sess.backward(want_du0=False)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.reps):
            g, _ = sess.backward(want_du0=False)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / (args.reps * args.adjoint)
        print(json.dumps({"N": args.N, "scheme": args.scheme, "adjoint_tiles": plan.adjoint_tiles(),
                          "tiles": plan.tiles(), "backward_step_ms": round(ms, 5),
                          "dJdtheta": [float(x) for x in g.cpu()]}))
        return
    flush = None if args.no_flush else torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    st = _native.time_stages(u0, th, L, 1e-4, 2.5e-4, args.scheme, args.reps, flush)
    try:
        with open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                               "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["hbm_gbs"])
    except Exception:
        peak = 6800.0
    out = {"N": args.N, "scheme": args.scheme, "tiles": plan.tiles(), "radix": plan.fft_radix(),
           "fused_rows": plan.fused_rows(), "stages": {}}
    for k, ms in st.items():
        gbs = _native.STAGE_BYTES_PER_CELL[k] * args.N * args.N / (ms * 1e-3) / 1e9
        out["stages"][k] = {"ms": round(ms, 5), "GB/s": round(gbs, 1), "frac": round(gbs / peak, 3)}
    out["step_ms"] = round(sum(st.values()), 5)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
