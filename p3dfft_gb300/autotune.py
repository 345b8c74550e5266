"""Autotuner for batched transforms.

Per grid shape and precision it picks the two plan knobs of
``p3g_plan_create_tuned`` -- the largest power-of-two radix of the FFT
stages (the radix split) and the cap on lines per shared-memory tile (the
tile shape) -- by timing round trips of that shape through the batch kernel
(captured CUDA graph, CUDA events).  Per batch it picks the queue window
(the transpose schedule: how many jobs run their X, Y and Z passes together;
see p3g_batch.cu).  Results are cached in a JSON file keyed by device name,
precision and shape (``P3G_TUNE_CACHE``, default
``~/.cache/p3dfft_gb300/tune.json``).

The reference leaves these choices to FFTW's planner (init_plan.F90:29-489,
FFTW_MEASURE); this tuner plays that role for the GPU kernels.
"""
from __future__ import annotations

import json
import os
import threading

from . import F32, F64, JOB_ROUNDTRIP, Batch, Plan

CACHE_ENV = "P3G_TUNE_CACHE"
WINDOWS = (1, 2, 4, 8, 16, 0)
_lock = threading.Lock()


def candidates(precision):
    """(max_radix, max_lines) pairs tried per shape; the first is the default."""
    if precision == F64:
        return [(8, 0), (4, 0), (8, 16), (8, 4)]
    return [(16, 0), (8, 0), (16, 16), (16, 4)]


def _cache_path() -> str:
    p = os.environ.get(CACHE_ENV)
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "p3dfft_gb300", "tune.json")


def _load() -> dict:
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def _key(shape, precision) -> str:
    import torch
    dev = torch.cuda.get_device_name().replace(" ", "_")
    return f"{dev}|{'f64' if precision == F64 else 'f32'}|{shape[0]}x{shape[1]}x{shape[2]}"


def time_batch(batch: Batch, reps: int = 5, warmup: int = 2, stream=None) -> float:
    """Milliseconds per replay of the batch's captured graph."""
    import torch
    stream = stream or torch.cuda.current_stream()
    batch.capture()
    for _ in range(warmup):
        batch.replay(stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        batch.replay(stream)
    e1.record(stream)
    batch.check(stream)
    return e0.elapsed_time(e1) / reps


def _roundtrip_jobs(plans, x, rdt):
    import torch
    jobs = []
    for p in plans:
        out = torch.empty((p.nz, p.ny, p.nx), dtype=rdt, device=x.device)
        jobs.append({"plan": p, "kind": JOB_ROUNDTRIP, "in": x, "out": out})
    return jobs


def tune_shape(shape, precision, reps: int = 5, min_points: int = 1 << 24, use_cache: bool = True,
               cands=None) -> dict:
    """Best (max_radix, max_lines) for round trips of `shape` among `cands`
    (default: candidates(precision)); times several copies of the grid in one
    batch so that the GPU is filled."""
    import torch
    key = _key(shape, precision)
    if use_cache:
        with _lock:
            hit = _load().get(key)
        if hit:
            return hit
    nx, ny, nz = shape
    npts = nx * ny * nz
    copies = max(1, min(32, min_points // max(1, npts)))
    rdt = torch.float64 if precision == F64 else torch.float32
    x = torch.rand((nz, ny, nx), dtype=rdt, device="cuda") * 2 - 1
    results = []
    for mr, ml in (cands or candidates(precision)):
        try:
            plans = [Plan(nx, ny, nz, precision=precision, max_radix=mr, max_lines=ml)] * copies
        except Exception:  # a knob outside what this shape supports
            continue
        b = Batch(precision).set_jobs(_roundtrip_jobs(plans, x, rdt))
        ms = time_batch(b, reps=reps)
        b.close()
        plans[0].close()
        results.append((ms / copies, mr, ml))
    results.sort()
    best = {"max_radix": results[0][1], "max_lines": results[0][2], "ms": results[0][0],
            "tried": [[r[1], r[2], r[0]] for r in results]}
    if use_cache:
        with _lock:
            d = _load()
            d[key] = best
            _store(d)
    return best


def tuned_plan(shape, precision, tune: bool = True, **kw) -> Plan:
    """A Plan with the cached (or freshly tuned) knobs for `shape`."""
    if tune:
        t = tune_shape(shape, precision)
        mr, ml = t["max_radix"], t["max_lines"]
    else:
        mr, ml = 0, 0
    return Plan(*shape, precision=precision, max_radix=mr, max_lines=ml, **kw)


def tune_window(jobs, precision, windows=WINDOWS, reps: int = 5) -> tuple[int, dict]:
    """Fastest queue window for a list of batch jobs; returns (window, ms by window)."""
    times = {}
    for w in windows:
        if w > len(jobs):
            continue
        b = Batch(precision).set_jobs(jobs, window=w)
        times[w] = time_batch(b, reps=reps)
        b.close()
    best = min(times, key=times.get)
    return best, times


__all__ = ["candidates", "tune_shape", "tuned_plan", "tune_window", "time_batch", "F32", "F64"]
