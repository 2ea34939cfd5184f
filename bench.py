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
measured live with CUDA events between the kernels of back-to-back solver
steps (the conditions of the timed rollout; each kernel alone from a cold L2
is reported beside it); ``cpu_baseline`` times
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
    ap.add_argument("--workload", choices=["plain", "grad", "ensemble", "serve", "optimize"], default="plain",
                    help="plain: the headline N=4096 rollout (default); grad: N=1024 adjoint; "
                         "ensemble: 256 uneven solves; serve: Poisson-arrival serving; optimize: the "
                         "reference's optimiser study on the device")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: arrivals per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: seconds of arrivals")
    ap.add_argument("--grad-mode", choices=["batched", "workers"], default="batched",
                    help="serve: gradient requests batched in lock-step, or one per worker thread")
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
    """nvidia-smi samples every 50 ms while the timed region runs."""
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
                 "-lms", "50"], stdout=self.fh, stderr=subprocess.DEVNULL)
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
def cpu_baseline(w, target_s: float = 10.0) -> dict:
    """The float32 oracle (restatement of the reference algorithm) on the
    host: about `target_s` seconds of solver steps of the same N=4096 workload
    (step count from a timed warm-up step), FFTs on all host cores (scipy.fft
    workers)."""
    from oracle import ns_oracle as O
    cores = len(os.sched_getaffinity(0))
    O.set_fft_workers(cores)
    u0, th = w.u0(), w.theta()
    cfg = O.OracleConfig(N=w.N, L=w.L, nu=w.nu, dt=w.dt, steps=w.steps, scheme=w.scheme)
    t0 = time.perf_counter()
    O.rollout(u0, th, cfg, steps=1)
    sample_steps = int(max(2, min(40, target_s / max(time.perf_counter() - t0, 1e-3))))
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


def ncu_traffic(stage: str, N: int = 4096):
    """DRAM bytes (read + write) per launch of a stage's kernel at size N, from
    the committed ncu summaries: a line 'traffic <stage> <N> <bytes>' in a
    profiles/*.md file."""
    d = os.path.join(ROOT, "profiles")
    try:
        names = sorted(f for f in os.listdir(d) if f.endswith(".md"))
    except OSError:
        return None
    for name in names:
        with open(os.path.join(d, name)) as f:
            for line in f:
                parts = line.strip().strip("`").split()
                if len(parts) == 4 and parts[0] == "traffic" and parts[1] == stage and parts[2] == str(N):
                    return float(parts[3])
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


def plain_config(w, world: int) -> dict:
    """The workload description both arms print (same keys, same values)."""
    return {"workload": w.name, "N": w.N, "solver_steps_per_step": w.steps, "dt": w.dt, "nu": w.nu,
            "scheme": w.scheme, "L": "2pi", "u0": f"seeded spectral |k|<={w.K}",
            "theta": "[A,B,nu] within 20% of [1,0.5,nu]", "parallelism": f"replicas{world}",
            "l2": "working set ~470 MB > L2 (no flush needed)",
            "cell_steps_per_step": int(w.N * w.N * w.steps)}


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

    # end to end through the public API: pinned host u0 in, (J, u_final) out,
    # every step.  Pipelined as a client streaming solves would run it: step
    # k+1's inputs are uploaded and step k's result read back on a copy
    # stream while step k computes (double-buffered device inputs and host
    # outputs); the serial form (copy in, solve, copy out on one stream) is
    # reported beside it.
    e2e = None
    if not args.no_e2e:
        u0_host = torch.from_numpy(u0_np).pin_memory()
        th_host = torch.from_numpy(th_np).pin_memory()
        uf_host = [torch.empty_like(u0_host).pin_memory() for _ in range(2)]
        J_host = [torch.empty((), dtype=torch.float32).pin_memory() for _ in range(2)]
        d_u0 = [torch.empty(u0_host.shape, dtype=torch.float32, device=dev) for _ in range(2)]
        d_th = [torch.empty(th_host.shape, dtype=torch.float32, device=dev) for _ in range(2)]
        copy = torch.cuda.Stream(dev)
        ev_in = [torch.cuda.Event() for _ in range(2)]
        ev_free = [torch.cuda.Event() for _ in range(2)]

        def upload(b):
            with torch.cuda.stream(copy):
                copy.wait_event(ev_free[b])
                d_u0[b].copy_(u0_host, non_blocking=True)
                d_th[b].copy_(th_host, non_blocking=True)
                ev_in[b].record(copy)

        def e2e_pipelined(n):
            upload(0)
            for k in range(n):
                b = k & 1
                stream.wait_event(ev_in[b])
                Jd, ufd = solver.rollout(d_u0[b], d_th[b])
                ev_free[b].record(stream)
                done = torch.cuda.Event()
                done.record(stream)
                if k + 1 < n:
                    upload(b ^ 1)
                with torch.cuda.stream(copy):
                    copy.wait_event(done)
                    uf_host[b].copy_(ufd, non_blocking=True)
                    J_host[b].copy_(Jd, non_blocking=True)
                    ufd.record_stream(copy)
                    Jd.record_stream(copy)
            torch.cuda.synchronize(dev)

        def e2e_serial(n):
            for _ in range(n):
                ud = u0_host.to(dev, non_blocking=True)
                td = th_host.to(dev, non_blocking=True)
                Jd, ufd = solver.rollout(ud, td)
                J_host[0].copy_(Jd, non_blocking=True)
                uf_host[0].copy_(ufd, non_blocking=True)
            torch.cuda.synchronize(dev)

        e2e_pipelined(2)
        e2e_serial(1)
        res = {}
        for name, fn in (("pipelined", e2e_pipelined), ("serial", e2e_serial)):
            if dist is not None:
                dist.barrier()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            fn(args.steps)
            res[name] = max_over_ranks(dist, time.perf_counter() - t0, dev)
        if not (math.isfinite(float(J_host[0])) and math.isfinite(float(J_host[1]))):
            raise RuntimeError("non-finite objective in the end-to-end rollouts")
        e2e = {"value": cells * args.steps * world / res["pipelined"], "unit": UNIT,
               "h2d_bytes_per_step": int(u0_host.numel() * 4 + th_host.numel() * 4),
               "d2h_bytes_per_step": int(uf_host[0].numel() * 4 + 4),
               "mode": "pipelined: each step's inputs uploaded from pinned host memory and its result read "
                       "back on a copy stream, overlapping the neighbouring steps' compute",
               "serial_value": cells * args.steps * world / res["serial"]}

    result = None
    if rank == 0:
        # per-kernel device times inside back-to-back solver steps (as in the
        # timed rollout), and each kernel alone from a cold L2
        st = _native.time_step_pipeline(u0, th, w.L, w.nu, w.dt, w.scheme, steps=20)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
        st_cold = _native.time_stages(u0, th, w.L, w.nu, w.dt, w.scheme, reps=10, flush=flush)
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
                    "launch_ms": round(st[dom], 5), "timing": "in-pipeline (CUDA events between the step kernels)",
                    "stages_ms": {k: round(v, 5) for k, v in st.items()},
                    "stage_share": {k: round(v, 3) for k, v in share.items()},
                    "cold_stages_ms": {k: round(v, 5) for k, v in st_cold.items()},
                    "cold_frac": round(alg / (st_cold[dom] * 1e-3) / 1e9 / peak, 4),
                    "step_bytes_per_cell": sum(bytes_cell.values()),
                    "step_frac_of_32B_ideal": round(32.0 * value / world / (peak * 1e9), 4)}
        # the CPU baseline is timed at N=1 only: under torchrun the other
        # ranks would hold their GPUs at the final barrier meanwhile
        cpu = None if (args.no_cpu_baseline or world > 1) else cpu_baseline(w)
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": plain_config(w, world),
            "tiles": {k: tiles.get(k, 16) for k in ("tw", "th", "rows", "cols", "radix_rows", "radix_cols")},
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
    warm = max(1, min(args.warmup, 10))  # warm-up solver steps, bounded
    O.rollout(u0, th, cfg, steps=warm)
    steps = max(1, min(args.steps, 40))  # one solver step per bench step, bounded
    t0 = time.perf_counter()
    O.rollout(u0, th, cfg, steps=steps)
    el = time.perf_counter() - t0
    value = float(w.N) * w.N * steps / el
    sample = (f"{steps} solver steps of the N={w.N} {w.scheme} workload (of its {w.steps}) after {warm} "
              f"warm-up; float32 NumPy oracle, FFTs via scipy.fft on {cores} workers")
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": steps, "warmup": warm, "ms_per_step": el / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": plain_config(w, world), "host": "cpu",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ------------------------------------------------- the systems workloads
def run_grad(args):
    """Differentiation: dJ/dtheta by the discrete adjoint, N=1024, 1000 steps,
    dt=1e-3, nu=5e-4, upwind; time against the forward rollout and peak memory
    with checkpoints every 50 steps (recompute in the backward pass) and with
    the automatic policy (every state kept when the states fit in half the
    free HBM: 8.4 GB here, no recompute).  The gradient is compared with the
    float64 oracle's derivative at the same point (central differences with
    relative steps 1e-7 for A -- the forcing's wrap puts kinks in J(A) closer
    than 1e-3 A -- and 1e-3 for B and nu), read from the committed fixture
    tests/golden/grad_N1024_upwind.json."""
    import torch
    import ns_solver_jax_differential_distributed_gb300 as nsgb
    from ns_solver_jax_differential_distributed_gb300 import _build, autotune
    from ns_solver_jax_differential_distributed_gb300.workloads import GRAD_N1024 as w, GRAD_CHECKPOINT_EVERY
    _build.build()
    dev = torch.device("cuda", 0)
    autotune.tune(w.N, w.L, w.scheme, dev)
    solver = nsgb.SingleCoreNSSolver(nsgb.make_grid(w.N, w.L), nsgb.Phys(nu=w.nu, mu0=0.5, sigma0=0.1, C=1.0),
                                     nsgb.Time(dt=w.dt, steps=w.steps), w.scheme, device=dev,
                                     checkpoint_every=GRAD_CHECKPOINT_EVERY)
    u0 = torch.from_numpy(w.u0()).to(dev)
    th = torch.from_numpy(w.theta()).to(dev)
    reps = max(1, args.steps)

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()  # a call repeated with the same arguments replays as a graph from the second on
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            out = fn()
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps, out

    clocks = ClockSampler(0).start()
    torch.cuda.reset_peak_memory_stats(dev)
    t_fwd, (J, _) = timed(lambda: solver.rollout(u0, th))
    mem_fwd = torch.cuda.max_memory_allocated(dev)
    torch.cuda.reset_peak_memory_stats(dev)
    t_grad, (Jg, g) = timed(lambda: solver.gradient(u0, th))
    mem_grad = torch.cuda.max_memory_allocated(dev)
    solver_all = nsgb.SingleCoreNSSolver(nsgb.make_grid(w.N, w.L), nsgb.Phys(nu=w.nu, mu0=0.5, sigma0=0.1, C=1.0),
                                         nsgb.Time(dt=w.dt, steps=w.steps), w.scheme, device=dev)
    every_auto = solver_all._every()
    torch.cuda.reset_peak_memory_stats(dev)
    t_all, (_, g_all) = timed(lambda: solver_all.gradient(u0, th))
    mem_all = torch.cuda.max_memory_allocated(dev)
    batch = grad_batch_compare(dev, reps)
    clock_info = clocks.stop()
    g = g.double().cpu().numpy()
    ref = None
    try:
        with open(os.path.join(ROOT, "tests", "golden", "grad_N1024_upwind.json")) as f:
            fx = json.load(f)["fd64"]
        ref = [fx["1e-07"][0], fx["0.001"][1], fx["0.001"][2]]
    except (OSError, KeyError):
        pass
    return {"metric": "adjoint gradient time / forward time", "value": t_grad / t_fwd, "unit": "x",
            "higher_is_better": False,
            "config": {"workload": w.name, "N": w.N, "steps": w.steps, "dt": w.dt, "nu": w.nu,
                       "scheme": w.scheme, "L": "2pi", "u0": f"seeded spectral |k|<={w.K}",
                       "checkpoint_every": GRAD_CHECKPOINT_EVERY},
            "forward_ms": t_fwd, "gradient_ms": t_grad, "reps": reps,
            "forward_cell_steps_per_s": float(w.N) * w.N * w.steps / (t_fwd / 1e3), "J": float(Jg),
            "dJdtheta": g.tolist(), "float64_derivative": ref,
            "rel_err_vs_float64": None if ref is None else [abs(a - b) / abs(b) for a, b in zip(g, ref)],
            "peak_mem_forward_bytes": mem_fwd, "peak_mem_gradient_bytes": mem_grad,
            "auto_checkpoint": {"checkpoint_every": every_auto, "gradient_ms": t_all,
                                "ratio_to_forward": t_all / t_fwd, "peak_mem_gradient_bytes": mem_all,
                                "max_abs_diff_vs_every_50": float(np.abs(g_all.double().cpu().numpy() - g).max())},
            "batched_gradients": batch,
            "clocks": clock_info, "dtype": "f32", "data": "synthetic"}


def grad_batch_compare(dev, reps: int, count: int = 16, seed: int = 5) -> dict:
    """`count` gradient requests drawn like the serving trace's small and
    mid sizes (N uniform over {128, 256, 512}, steps U[100, 400], upwind,
    the stable time step, checkpoints every 50): solved one after another by
    nsgb_rollout_grad, and together by nsgb_grad_batch_advance (lock-step,
    one batched launch per kernel per size group).  Both are timed with CUDA
    events on the device (host gaps included); results must agree bit for
    bit."""
    import torch
    from ns_solver_jax_differential_distributed_gb300 import _native, autotune, ensemble, serve
    from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0, theta_draw
    L = 2 * math.pi
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        N = int(rng.choice([128, 256, 512]))
        steps = int(rng.integers(100, 401))
        th = theta_draw(1e-3, seed=i)
        nu = float(th[2])
        reqs.append(dict(N=N, steps=steps, nu=nu, dt=serve.stable_dt(N, L, nu),
                         u0=torch.from_numpy(spectral_u0(N, min(32, N // 4), i)).to(dev),
                         th=torch.from_numpy(th).to(dev)))
    for N in sorted({r["N"] for r in reqs}):
        autotune.tune(N, L, "upwind", dev)

    def sequential():
        return [_native.rollout_grad_raw(r["u0"], r["th"], r["steps"], 50, L, r["nu"], r["dt"], "upwind",
                                         want_u_final=False)[:2] for r in reqs]

    def batched():
        gb = ensemble.GradientBatch(dev)
        ids = [gb.add(r["u0"], r["th"], r["steps"], 50, L, r["nu"], r["dt"], "upwind") for r in reqs]
        gb.run(64)
        return [gb.result(k) for k in ids]

    def timed(fn):
        for _ in range(3):
            out = fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            out = [(J.clone(), g.clone()) for J, g in fn()]
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps, out

    t_seq, out_seq = timed(sequential)
    t_bat, out_bat = timed(batched)
    same = all(torch.equal(a[0], b[0]) and torch.equal(a[1], b[1]) for a, b in zip(out_seq, out_bat))
    sizes = {}
    for r in reqs:
        sizes[str(r["N"])] = sizes.get(str(r["N"]), 0) + 1
    return {"requests": count, "sizes": sizes, "steps": "U[100,400]", "checkpoint_every": 50,
            "sequential_ms": t_seq, "batched_ms": t_bat, "speedup": t_seq / t_bat,
            "results_bitwise_equal": bool(same), "reps": reps}


def run_optimize(args):
    """The reference's parameter optimisation study (studies.py:864-934):
    Adam (lr 0.01, 0.001), SGD (lr 0.1), RMSprop (lr 0.01), 100 steps each
    from theta0 = [1, 0.5], objective from the zero state at N=128, L=1,
    nu=0.01, 328 steps (SimConfig's dt), central -- each optimiser one
    nsgb_optimize call.  Reports device time per optimiser step (one adjoint
    gradient + update) and the final objectives; the reference's CPU run of
    the same study takes 0.119 s per jit_gradient call (BASELINE)."""
    import torch
    import ns_solver_jax_differential_distributed_gb300 as nsgb
    from ns_solver_jax_differential_distributed_gb300 import _build, autotune, optimization
    _build.build()
    dev = torch.device("cuda", 0)
    N, L, nu, steps = 128, 1.0, 0.01, 328
    dt = float(np.float32(min(0.4 * (L / N), (L / N) ** 2 / (4 * nu))))
    autotune.tune(N, L, "central", dev)
    solver = nsgb.SingleCoreNSSolver(nsgb.make_grid(N, L), nsgb.Phys(nu=nu, mu0=0.5, sigma0=0.1, C=1.0),
                                     nsgb.Time(dt=dt, steps=steps), "central", device=dev)
    study = optimization.ParameterOptimizationStudy(solver.jit_objective, solver.jit_gradient, [1.0, 0.5],
                                                    optim_steps=100)
    study.run_all()  # warm-up (plans, workspaces)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0).start()
    t0 = time.perf_counter()
    e0.record()
    res = study.run_all()
    e1.record()
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    clock_info = clocks.stop()
    n_steps = 4 * 100
    return {"metric": "optimiser steps/s", "value": n_steps / (e0.elapsed_time(e1) / 1e3), "unit": "steps/s",
            "higher_is_better": True, "ms_per_optimizer_step": e0.elapsed_time(e1) / n_steps,
            "wall_s": wall, "clocks": clock_info,
            "config": {"workload": "optimiser study (studies.py:864-934)", "N": N, "L": L, "nu": nu, "dt": dt,
                       "steps": steps, "scheme": "central",
                                       "theta0": [1.0, 0.5], "optim_steps": 100,
                                       "checkpoint_every": solver._every()},
            "final": {k: {"obj_initial": v["obj_initial"], "obj_final": v["obj_final"],
                          "improvement": v["improvement"],
                          "theta_final": np.asarray(v["history"]["parameters"][-1]).tolist()}
                      for k, v in res.items()},
            "reference_cpu_s_per_gradient": 0.119, "dtype": "f32", "data": "synthetic"}


def sizes_of(members):
    return sorted({m.N for m in members})


def run_ensemble(args):
    """Batching: 256 solves, N in {64,128,256,512} w.p. {.4,.3,.2,.1}, 500
    steps, per-solve nu/theta/u0; one batched launch per stage per N-group,
    CUDA-graph chunks of 16 steps, stencil shapes tuned for the batch; against
    256 sequential plain rollouts with single-solve tuned shapes."""
    import torch
    from ns_solver_jax_differential_distributed_gb300 import _build, ensemble
    from ns_solver_jax_differential_distributed_gb300.workloads import ensemble as make_ensemble
    _build.build()
    dev = torch.device("cuda", 0)
    members = make_ensemble()
    specs = ensemble.from_workload(members)
    # single-solve launch shapes for the sequential comparison, then the
    # batch-tuned shapes for the batched run
    from ns_solver_jax_differential_distributed_gb300 import autotune
    for N in sorted({m.N for m in members}):
        autotune.tune(N, members[0].L, "central", dev)
    ens = ensemble.Ensemble(specs, steps=members[0].steps, device=dev, chunk=16)

    def timed(fn):
        fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(max(1, args.steps)):
            out = fn()
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / max(1, args.steps), out

    clocks = ClockSampler(0).start()
    t_s, (Js, us) = timed(ens.run_sequential)
    Js, us = Js.clone(), [u.clone() for u in us]
    seq_clocks = clocks.stop()
    ens.tune_batched()
    clocks = ClockSampler(0).start()
    t_b, (Jb, ub) = timed(ens.run)
    Jb, ub = Jb.clone(), [u.clone() for u in ub]
    # the same ensemble in one persistent cooperative launch (stencil tiles
    # 32 x 8, radix-16 transforms)
    t_p, (Jp, up) = timed(ens.run_persistent)
    clock_info = clocks.stop()
    radix16 = all(tuple(ensemble._native.get_plan(N, members[0].L, dev).fft_radix()) == (16, 16)
                  for N in sizes_of(members))
    pers = {"ms": t_p, "cell_steps_per_s": float(ens.cell_steps) / (t_p / 1e3),
            "solves_per_s": len(members) / (t_p / 1e3), "vs_batched": t_b / t_p,
            "fields_bitwise_equal_to_batched": all(torch.equal(a, b) for a, b in zip(up, ub)),
            "plans_radix16": radix16,
            "max_abs_field_diff": max(float((a - b).abs().max()) for a, b in zip(up, ub))}
    # fields are bit-identical across launch shapes; J sums per-block
    # partials, whose grouping follows the shape
    same = all(torch.equal(a, b) for a, b in zip(ub, us))
    finite = sum(bool(torch.isfinite(u).all()) and math.isfinite(float(j)) for u, j in zip(ub, Jb))
    j_rel = float(((Jb.double() - Js.double()).abs() / Js.double().abs().clamp_min(1e-30)).max())
    cells = float(ens.cell_steps)
    sizes = {}
    for m in members:
        sizes[m.N] = sizes.get(m.N, 0) + 1
    return {"metric": "batched cell-steps/s", "value": cells / (t_b / 1e3), "unit": "cell-steps/s",
            "sequential_cell_steps_per_s": cells / (t_s / 1e3), "speedup_vs_sequential": t_s / t_b,
            "solves_per_s_batched": len(members) / (t_b / 1e3),
            "solves_per_s_sequential": len(members) / (t_s / 1e3),
            "speedup_vs_plain": t_s / t_b, "finite_members": finite,
            "batched_ms": t_b, "sequential_ms": t_s, "fields_bitwise_equal_to_sequential": same, "J_max_rel_diff": j_rel,
            "members": len(members), "sizes": sizes, "steps": members[0].steps, "dtype": "f32",
            "config": {"workload": "ensemble of 256 uneven solves", "sizes": "N in {64,128,256,512} w.p. "
                       "{.4,.3,.2,.1}", "steps": members[0].steps, "dt": members[0].dt,
                       "nu": "log-uniform [1e-4, 1e-2]", "theta": "within 20% of default, per solve",
                       "plain": "256 sequential single-solve rollouts (single-solve tuned shapes)"},
            "persistent_launch": pers,
            "clocks": clock_info, "clocks_sequential": seq_clocks,
            "data": "synthetic", "chunk": 16}


def plain_serve(reqs, dev, budget_s: float):
    """The same requests solved one at a time through the plain per-request
    API (a rollout, or a checkpointed adjoint gradient, per request; the
    result read back before the next starts), in arrival order, for about
    `budget_s` seconds: the throughput of serving without batching or
    overlap."""
    import torch
    from ns_solver_jax_differential_distributed_gb300 import _native, serve
    u0s = serve._U0Cache(dev)
    n, t0 = 0, time.perf_counter()
    for r in reqs:
        if time.perf_counter() - t0 > budget_s:
            break
        u0 = u0s.get(r.N, r.seed)
        th = torch.from_numpy(r.theta).to(dev)
        if r.kind == "grad":
            J, g, _, _ = _native.rollout_grad_raw(u0, th, r.steps, 50, r.L, r.nu, r.dt, r.scheme,
                                                  want_u_final=False, own_workspace=True)
            float(J), g.cpu()
        else:
            J, u = _native.op_rollout(u0, th, r.steps, r.L, r.nu, r.dt, _native.SCHEME_IDS[r.scheme],
                                      0.5, 0.1, 1.0, True)
            float(J)
        n += 1
    wall = time.perf_counter() - t0
    return {"solves": n, "wall_s": wall, "solves_per_s": n / wall}


def run_serve(args):
    """Serving: Poisson arrivals at --rate for --duration s; N uniform over
    {128..2048}, steps U[100,2000], 30% forward+adjoint; 150 GB HBM budget;
    continuous batching.  Reports solves/s and p50/p99 latency; the run stops
    30 s after the last arrival (requests still queued are reported).  The
    same trace's requests, solved one by one through the plain per-request
    API for about 30 s, give the plain throughput the served one is compared
    with."""
    import torch
    from ns_solver_jax_differential_distributed_gb300 import _build, serve, autotune
    _build.build()
    dev = torch.device("cuda", 0)
    for N in (128, 256, 512, 1024, 2048):
        autotune.tune(N, 2 * math.pi, "upwind", dev)
    reqs = serve.make_trace(rate=args.rate, duration=args.duration, seed=7)
    srv = serve.Server(dev, hbm_budget=150e9, grad_mode=args.grad_mode)
    for N in (128, 256, 512, 1024, 2048):
        for s in range(16):
            srv.u0.get(N, s)
    plain_serve(reqs[:8], dev, 5.0)  # warm-up: plans, workspaces, graphs
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(0).start()
    t0 = time.perf_counter()
    done, trace = srv.run(reqs, realtime=True, drain_limit=30.0, suspend=False)
    wall = time.perf_counter() - t0
    clock_info = clocks.stop()
    summ = serve.summarize(reqs, done, wall)
    clocks = ClockSampler(0).start()
    plain = plain_serve(serve.make_trace(rate=args.rate, duration=args.duration, seed=7), dev, 30.0)
    plain["clocks"] = clocks.stop()
    summ.update({"metric": "served solves/s", "rate_req_per_s": args.rate, "duration_s": args.duration,
                 "max_queue": max(q[1] for q in trace) if trace else 0,
                 "queue_at_end": trace[-1][1] if trace else 0,
                 "grad_fraction_completed": (sum(r.kind == "grad" for r in done if r.status == "ok")
                                             / max(1, sum(r.status == "ok" for r in done))),
                 "plain_per_request": plain,
                 "speedup_vs_plain": summ["solves_per_s"] / plain["solves_per_s"],
                 "clocks": clock_info,
                 "config": {"workload": "serving", "arrivals": f"Poisson {args.rate} req/s for {args.duration} s",
                            "N": "uniform over {128,256,512,1024,2048}", "steps": "U[100,2000]",
                            "grad_fraction": 0.3, "hbm_budget_bytes": 150e9, "scheme": "upwind",
                            "dt": "stable step of each request's N and nu (cfl 0.4, v_max 4)",
                            "grad_mode": args.grad_mode, "grad_checkpoint_every": serve.GRAD_EVERY}})
    return summ


def main(argv=None):
    args = parse_args(argv)
    world, rank, local = dist_env()
    if args.workload != "plain":
        if rank == 0:
            fn = {"grad": run_grad, "ensemble": run_ensemble, "serve": run_serve,
                  "optimize": run_optimize}[args.workload]
            print(json.dumps(fn(args)), flush=True)
        return
    if args.impl == "reference":
        res = run_reference(args, world, rank)
    else:
        res = run_ours(args, world, rank, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
