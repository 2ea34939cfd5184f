#!/usr/bin/env python
"""Benchmark of the GB300 Chorin-projection solver.

Workload (one bench "step"): one full rollout of the headline configuration
-- N=4096 on [0, 2 pi]^2, float32, 200 solver steps, dt=2.5e-4, nu=1e-4,
central advection (``--scheme upwind`` for the other run), seeded spectral u0
(|k| <= 32) and a seeded 3-entry theta.  Metric: cell-steps/s = N^2 * 200 /
rollout time.  The working set (about 470 MB) is larger than L2, so no flush
is needed between timed rollouts.

Output: one JSON line (rank 0).  ``value`` is device-timed with inputs
resident in HBM; ``e2e`` is the same metric through the public API with the
initial state copied from pinned host memory and (J, u_final) read back every
step; ``roofline`` is the dominant kernel's achieved HBM bandwidth, its time
measured live with CUDA events (cold L2 per launch); ``cpu_baseline`` times
the float32 CPU oracle (a restatement of the reference algorithm; JAX is not
available) on a bounded sample.

``--gpus N`` under torchrun runs N independent replicas (one solve per GPU,
no collective on the data path): weak scaling.  ``--impl reference`` times the
reference algorithm's CPU implementation (the oracle port) instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "cell-steps/s"
UNIT = "cell-steps/s"
FALLBACK_HBM_GBS = 6800.0


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10, help="timed rollouts")
    ap.add_argument("--warmup", type=int, default=3, help="untimed rollouts (>= 3)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scheme", choices=["central", "upwind"], default="central")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args(argv)


# ------------------------------------------------------------- distributed
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init_dist(world: int, backend: str):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(dist, x: float, device=None) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- CPU baseline
def cpu_baseline(w, sample_steps: int = 2) -> dict:
    """The float32 oracle (restatement of the reference algorithm) on the
    host: `sample_steps` solver steps of the same N=4096 workload after one
    warm-up step, FFTs on all host cores (scipy.fft workers)."""
    from oracle import ns_oracle as O
    cores = len(os.sched_getaffinity(0))
    O.set_fft_workers(cores)
    u0, th = w.u0(), w.theta()
    cfg = O.OracleConfig(N=w.N, L=w.L, nu=w.nu, dt=w.dt, steps=w.steps, scheme=w.scheme)
    O.rollout(u0, th, cfg, steps=1)
    t0 = time.perf_counter()
    O.rollout(u0, th, cfg, steps=sample_steps)
    dt_s = time.perf_counter() - t0
    O.set_fft_workers(None)
    return {"value": w.N * w.N * sample_steps / dt_s, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{sample_steps} solver steps of the N={w.N} {w.scheme} workload after 1 warm-up "
                      f"step ({dt_s:.1f} s); float32 NumPy oracle, FFTs via scipy.fft with {cores} workers"}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (a line 'traffic <kernel> <N> <bytes>' in profiles/ncu_summary.md)."""
    path = os.path.join(ROOT, "profiles", "ncu_summary.md")
    try:
        with open(path) as f:
            for line in f:
                parts = line.strip().strip("`").split()
                if len(parts) == 4 and parts[0] == "traffic" and parts[1] == kernel and parts[2] == "4096":
                    return float(parts[3])
    except OSError:
        pass
    return None


def launches_per_rollout(steps: int, use_graph: bool, chunk: int = 16) -> int:
    """Kernels of libnsgb one rollout launches (4 per solver step, the
    chunk-graph step counter, the final projection and the J reduction)."""
    if steps == 0:
        return 1
    n = 4 * steps + 1 + 2
    if use_graph and steps - 1 >= 2 * chunk:
        n += 1 + (steps - 1) // chunk
    return n


# --------------------------------------------------------------- our arm
def run_ours(args, world, rank, local):
    import torch
    from ns_solver_jax_differential_distributed_gb300 import _build, _native
    import ns_solver_jax_differential_distributed_gb300 as nsgb
    from ns_solver_jax_differential_distributed_gb300.workloads import (
        PLAIN_SCALE_CENTRAL, PLAIN_SCALE_UPWIND)

    _build.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = init_dist(world, "nccl")
    w = PLAIN_SCALE_CENTRAL if args.scheme == "central" else PLAIN_SCALE_UPWIND
    from ns_solver_jax_differential_distributed_gb300 import autotune
    tiles = autotune.tune(w.N, w.L, w.scheme, dev)  # cached after the first run on a GPU
    grid = nsgb.make_grid(w.N, w.L)
    phys = nsgb.Phys(nu=w.nu, mu0=0.5, sigma0=0.1, C=1.0)
    solver = nsgb.SingleCoreNSSolver(grid, phys, nsgb.Time(dt=w.dt, steps=w.steps), w.scheme,
                                     device=dev, use_graph=True)
    u0_np, th_np = w.u0(), w.theta()
    u0 = torch.from_numpy(u0_np).to(dev)
    th = torch.from_numpy(th_np).to(dev)
    stream = torch.cuda.current_stream(dev)

    warm = max(3, args.warmup)
    for _ in range(warm):
        J, uf = solver.rollout(u0, th)
    torch.cuda.synchronize(dev)

    clocks = ClockSampler(local).start() if rank == 0 else None
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        J, uf = solver.rollout(u0, th)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    if dist is not None:
        dist.barrier()
    elapsed_ms = max_over_ranks(dist, e0.elapsed_time(e1), dev)
    clock_info = clocks.stop() if clocks else None
    if not math.isfinite(float(J)):
        raise RuntimeError("non-finite objective in the benchmark rollout")
    cells = float(w.N) * w.N * w.steps
    value = cells * args.steps * world / (elapsed_ms / 1e3)
    ms_per_step = elapsed_ms / args.steps

    # end to end through the public API: pinned host u0 in, (J, u_final) out
    e2e = None
    if not args.no_e2e:
        u0_host = torch.from_numpy(u0_np).pin_memory()
        th_host = torch.from_numpy(th_np).pin_memory()
        uf_host = torch.empty_like(u0_host).pin_memory()
        J_host = torch.empty((), dtype=torch.float32).pin_memory()

        def e2e_step():
            ud = u0_host.to(dev, non_blocking=True)
            td = th_host.to(dev, non_blocking=True)
            Jd, ufd = solver.rollout(ud, td)
            J_host.copy_(Jd, non_blocking=True)
            uf_host.copy_(ufd, non_blocking=True)

        e2e_step()
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize(dev)
        e2e_s = max_over_ranks(dist, time.perf_counter() - t0, dev)
        e2e = {"value": cells * args.steps * world / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(u0_host.numel() * 4 + th_host.numel() * 4),
               "d2h_bytes_per_step": int(uf_host.numel() * 4 + 4)}

    result = None
    if rank == 0:
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
        st = _native.time_stages(u0, th, w.L, w.nu, w.dt, w.scheme, reps=10, flush=flush)
        del flush
        bytes_cell = _native.STAGE_BYTES_PER_CELL
        share = {k: v / sum(st.values()) for k, v in st.items()}
        dom = max(st, key=st.get)
        peak, peak_kind = measured_peak()
        alg = bytes_cell[dom] * float(w.N) * w.N
        achieved = alg / (st[dom] * 1e-3) / 1e9
        roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                    "peak_source": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                    "traffic": ncu_traffic(dom), "algorithmic_bytes_per_launch": alg,
                    "launch_ms": round(st[dom], 5),
                    "stages_ms": {k: round(v, 5) for k, v in st.items()},
                    "stage_share": {k: round(v, 3) for k, v in share.items()},
                    "step_bytes_per_cell": sum(bytes_cell.values()),
                    "step_frac_of_32B_ideal": round(32.0 * value / world / (peak * 1e9), 4)}
        cpu = None if args.no_cpu_baseline else cpu_baseline(w)
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w.name, "N": w.N, "solver_steps_per_step": w.steps, "dt": w.dt,
                       "nu": w.nu, "scheme": w.scheme, "L": "2pi", "u0": f"seeded spectral |k|<={w.K}",
                       "theta": "[A,B,nu] within 20% of [1,0.5,nu]", "parallelism": f"replicas{world}",
                       "l2": "working set ~470 MB > L2 (no flush needed)",
                       "tiles": {k: tiles[k] for k in ("tw", "th", "rows", "cols")},
                       "cell_steps_per_step": int(cells)},
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clock_info,
            "gpu_launches": launches_per_rollout(w.steps, True) * args.steps,
            "J": float(J),
        }
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return result


# --------------------------------------------------------- reference arm
def run_reference(args, world, rank):
    """The reference algorithm's CPU implementation (the float32 oracle port;
    JAX is not installed) on the same workload; each bench step is one solver
    step of the N=4096 rollout (a bounded sample)."""
    if rank != 0:
        return None
    from oracle import ns_oracle as O
    from ns_solver_jax_differential_distributed_gb300.workloads import (
        PLAIN_SCALE_CENTRAL, PLAIN_SCALE_UPWIND)
    w = PLAIN_SCALE_CENTRAL if args.scheme == "central" else PLAIN_SCALE_UPWIND
    cores = len(os.sched_getaffinity(0))
    O.set_fft_workers(cores)
    u0, th = w.u0(), w.theta()
    cfg = O.OracleConfig(N=w.N, L=w.L, nu=w.nu, dt=w.dt, steps=w.steps, scheme=w.scheme)
    warm = max(1, min(args.warmup, 2))
    O.rollout(u0, th, cfg, steps=warm)
    steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    O.rollout(u0, th, cfg, steps=steps)
    el = time.perf_counter() - t0
    value = float(w.N) * w.N * steps / el
    sample = (f"{steps} solver steps of the N={w.N} {w.scheme} workload (of its {w.steps}) after {warm} "
              f"warm-up; float32 NumPy oracle, FFTs via scipy.fft on {cores} workers")
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": steps, "warmup": warm, "ms_per_step": el / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w.name, "N": w.N, "scheme": w.scheme, "parallelism": "host cpu"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main(argv=None):
    args = parse_args(argv)
    world, rank, local = dist_env()
    if args.impl == "reference":
        res = run_reference(args, world, rank)
    else:
        res = run_ours(args, world, rank, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
