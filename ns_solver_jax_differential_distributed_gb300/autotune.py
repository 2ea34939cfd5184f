"""Launch-shape autotuner for the solver kernels.

For one (N, scheme, GPU) it times every valid candidate of each stage's launch
shape with CUDA events (``nsgb_time_stages``: mean device time per launch,
cold L2 for grids larger than L2) and keeps the fastest per stage:

* stencil launch shape: a tile (width x height cells) of the tiled kernel or
  a band (width x rows) of the row-streaming kernel,
* Stockham radix (16 or 8) and rows per CTA of the row FFTs (forward and
  inverse),
* Stockham radix and spectrum rows per CTA of the column FFT.

Results are cached in a JSON file keyed by GPU name, N and scheme
(``$NSGB_TUNE_CACHE`` or ``<package>/_autotune/tiles.json``) so a process
tunes a size once.  The stages are independent kernels, so each shape is
tuned separately.
"""
from __future__ import annotations

import json
import math
import os
import threading

import torch

from . import _native

_CACHE_PATH = os.environ.get("NSGB_TUNE_CACHE") or os.path.join(
    os.path.dirname(os.path.abspath(__file__)), "_autotune", "tiles.json")
_lock = threading.Lock()

# the shapes csrc/nsgb_common.cuh instantiates (NSGB_STENCIL_TILES)
STENCIL_TILES = [(16, 8), (16, 16), (32, 8), (32, 16), (64, 8), (64, 16), (128, 8)]
ROW_CHOICES = [2, 4, 8, 16]
COL_CHOICES = [1, 2, 4]
RADIX_CHOICES = [16, 8]


def _load() -> dict:
    try:
        with open(_CACHE_PATH) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(data: dict) -> None:
    # Several processes (one per GPU under torchrun) may tune at once: each
    # writes its own temporary file and renames it over the cache, so every
    # version of the cache on disk is complete (the last writer's entries win).
    os.makedirs(os.path.dirname(_CACHE_PATH), exist_ok=True)
    tmp = f"{_CACHE_PATH}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, _CACHE_PATH)


def _key(N: int, scheme: str, device) -> str:
    return f"{torch.cuda.get_device_name(device)}|N={N}|{scheme}"


# Row-streaming stencil: band widths (min(width, N) columns per CTA) and the
# CTA counts per SM the row bands are sized for.
ROW_BAND_WIDTHS = [256, 512, 1024, 2048]
ROW_BAND_WAVES = [1, 2, 3, 4]


def row_band_shapes(N: int, sms: int) -> list:
    """(width, rows) shapes of the row-streaming stencil worth timing for N:
    each distinct band width, with the row counts that give about 1-4 CTAs
    per SM (at least 8 rows: a band recomputes 4 rows of its neighbours)."""
    out = []
    for W in sorted({min(w, N) for w in ROW_BAND_WIDTHS}):
        col_bands = N // W
        for waves in ROW_BAND_WAVES:
            bands = max(1, -(-waves * sms // col_bands))
            rows = min(N, max(8, -(-N // bands)))
            if (W, rows) not in out:
                out.append((W, rows))
    return out


# widest band of the row-streaming adjoint kernel
ADJ_ROWS_MAX_W = 1024


def candidates(N: int, sms: int = 152) -> dict:
    st = [(w, h) for (w, h) in STENCIL_TILES if w <= N and h <= N]
    adj = list(st)
    if N >= 256:
        st += row_band_shapes(N, sms)
        adj += [(w, h) for (w, h) in row_band_shapes(N, sms) if w <= ADJ_ROWS_MAX_W]
    rows, cols = [], []
    for radix in RADIX_CHOICES:
        T = N // min(radix, N)
        rows += [(radix, r) for r in ROW_CHOICES if r <= N and (r // 2) * T <= 1024]
        cols += [(radix, c) for c in COL_CHOICES if c <= N // 2 and c * T <= 512]
    return {"stencil": st, "rows": rows, "cols": cols, "adjoint": adj}


def _apply(plan, best: dict) -> None:
    # radix first at shapes valid for both radices, then the tuned shapes
    plan.set_tiles(best["tw"], best["th"], 2, 1)
    plan.set_fft_radix(best.get("radix_rows", 16), best.get("radix_cols", 16))
    plan.set_tiles(best["tw"], best["th"], best["rows"], best["cols"])
    if "adj_tw" in best:
        plan.set_adjoint_tiles(best["adj_tw"], best["adj_th"])


def _time_adjoint(u0, th, L, nu, dt, scheme, reps: int, steps: int = 6) -> float:
    """Mean device ms of one backward step (adjoint stencil + FFT passes),
    every state stored (no recompute)."""
    sess = _native.GradSession(u0, th, steps, 1, L, nu, dt, scheme)
    sess.forward()
    for _ in range(2):  # the second identical call captures the graph later calls replay
        sess.backward(want_du0=False)
    torch.cuda.synchronize(u0.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        sess.backward(want_du0=False)
    e1.record()
    torch.cuda.synchronize(u0.device)
    return e0.elapsed_time(e1) / (reps * steps)


def tune(N: int, L: float = 2 * math.pi, scheme: str = "central", device=None, reps: int = 5,
         force: bool = False, verbose: bool = False) -> dict:
    """Tune and apply the launch shapes of the plan (N, L, device)."""
    device = torch.device(device or "cuda")
    plan = _native.get_plan(N, L, device)
    key = _key(N, scheme, device)
    with _lock:
        cache = _load()
        if key in cache and not force:
            best = cache[key]
            _apply(plan, best)
            return best
    from .workloads import spectral_u0
    u0 = torch.from_numpy(spectral_u0(N, min(32, N // 4), 0)).to(device)
    th = torch.tensor([1.0, 0.5, 1e-3], device=device)
    dt, nu = 1e-4, 1e-3
    cells = N * N
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device) if cells * 28 > (96 << 20) else None
    cand = candidates(N, torch.cuda.get_device_properties(device).multi_processor_count)
    base = plan.tiles()
    base_radix = plan.fft_radix()
    results = {"stencil": {}, "rows": {}, "cols": {}}
    for (w, h) in cand["stencil"]:
        plan.set_tiles(w, h, base[2], base[3])
        results["stencil"][(w, h)] = _native.time_stages(u0, th, L, nu, dt, scheme, reps, flush)["stencil"]
    # FFT shapes: each (radix, CTA shape) of one pass with the other pass at
    # its smallest shape, which every radix accepts
    for (radix, r) in cand["rows"]:
        plan.set_tiles(base[0], base[1], 2, 1)
        plan.set_fft_radix(radix, 16)
        plan.set_tiles(base[0], base[1], r, 1)
        t = _native.time_stages(u0, th, L, nu, dt, scheme, reps, flush)
        results["rows"][(radix, r)] = t["rows_fwd"] + t["rows_inv"]
    for (radix, c) in cand["cols"]:
        plan.set_tiles(base[0], base[1], 2, 1)
        plan.set_fft_radix(16, radix)
        plan.set_tiles(base[0], base[1], 2, c)
        results["cols"][(radix, c)] = _native.time_stages(u0, th, L, nu, dt, scheme, reps, flush)["cols"]
    tw, thh = min(results["stencil"], key=results["stencil"].get)
    rr, rows = min(results["rows"], key=results["rows"].get)
    rc, cols = min(results["cols"], key=results["cols"].get)
    best = {"tw": tw, "th": thh, "rows": rows, "cols": cols, "radix_rows": rr, "radix_cols": rc,
            "ms": {"stencil": results["stencil"][(tw, thh)], "rows_fwd+inv": results["rows"][(rr, rows)],
                   "cols": results["cols"][(rc, cols)]},
            "default": list(base) + list(base_radix)}
    _apply(plan, best)
    # adjoint shapes: one backward step with the tuned FFT shapes
    results["adjoint"] = {}
    base_adj = plan.adjoint_tiles()
    for (w, h) in cand["adjoint"]:
        plan.set_adjoint_tiles(w, h)
        results["adjoint"][(w, h)] = _time_adjoint(u0, th, L, nu, dt, scheme, max(2, reps // 2))
    best["adj_tw"], best["adj_th"] = min(results["adjoint"], key=results["adjoint"].get)
    best["ms"]["adjoint_step"] = results["adjoint"][(best["adj_tw"], best["adj_th"])]
    best["default"] += list(base_adj)
    plan.set_adjoint_tiles(best["adj_tw"], best["adj_th"])
    if verbose:
        print(f"autotune N={N} {scheme}: best {best}")
        for kind, res in results.items():
            print(f"  {kind}: " + ", ".join(f"{k}={v * 1e3:.1f}us" for k, v in sorted(res.items(), key=lambda kv: kv[1])))
    with _lock:
        cache = _load()
        cache[key] = best
        _store(cache)
    return best


def apply_cached(N: int, L: float, scheme: str, device=None) -> bool:
    """Apply cached shapes if present (no timing); True if applied."""
    device = torch.device(device or "cuda")
    best = _load().get(_key(N, scheme, device))
    if not best:
        return False
    _apply(_native.get_plan(N, L, device), best)
    return True
