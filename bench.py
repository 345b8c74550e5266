"""Benchmark of the P3DFFT 3D r2c + c2r transform path on GB300.

One step = one forward r2c ('fft') plus one backward c2r ('tff') of one
synthetic grid (the reference sample drivers' timed loop,
sample/FORTRAN/driver_rand.F90:209-243).  The headline workload is the
1024^3 FP64 round trip; the line also carries the FP32 form on the same grid.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config large|noncubic|small|cheby]
  python bench.py --impl reference ...   # the CPU reference arm (oracle port, all host cores)

Under torchrun (N > 1) every rank runs an independent replica of the
workload on its own GPU (the path does not shard on one GPU per rank):
value = points of all ranks / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "3D r2c+c2r Gpts/s & %HBM roofline, FP32 vs FP64 at stated error; serve p50/p99"
UNIT = "Gpts/s"

CONFIGS = {
    "large": dict(grid=(1024, 1024, 1024), ops=("fft", "tff"), input="modes",
                  workload="1024^3 FP64 r2c+c2r round trip (32 seeded Fourier modes + N(0,1e-3) noise)"),
    "noncubic": dict(grid=(768, 1024, 540), ops=("fft", "tff"), input="modes",
                     workload="768x1024x540 FP64 r2c+c2r round trip (32 seeded Fourier modes + N(0,1e-3) noise)"),
    "small": dict(grid=(128, 128, 128), ops=("fft", "tff"), input="uniform",
                  workload="128^3 FP64 r2c+c2r round trip, U[-1,1)"),
    "cheby": dict(grid=(512, 512, 257), ops=("ffc", "cff"), input="cheby",
                  workload="512x512x257 FP64 FFT(x,y) + DCT-I(z) round trip, 16 seeded sin cos T_m(z) terms "
                           "on Gauss-Lobatto z + 1e-6 noise; p3dfft_cheby beside it"),
}


MODES = {"pipe_tma": (True, True), "pipe_cpasync": (True, False), "single_tile": (False, False)}

# DRAM bytes (read + write) per algorithmic byte of one launch of the
# dominant kernel, from ncu captures of its Y pass on a 1024x1024x32 grid
# (273.69 MB read + 225.91 MB written) and its Z passes on a 1024x32x1024
# grid (273.93 + 222.29 and 270.01 + 224.63 MB), each for 538.97 MB of 2C
# model traffic; the four launches of a round trip (Y, Z, Z, Y) averaged.
# The full-size launches move the same bytes per line, so traffic scales
# with the model.
TRAFFIC_PER_ALGO_BYTE = {
    "k_strided_pipe": (2 * (273.687040e6 + 225.914880e6) + (273.926656e6 + 222.291712e6) +
                       (270.008320e6 + 224.634880e6)) / (4 * 538968064.0)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------- inputs
def modes_list(grid, seed, count=32):
    """The seeded Fourier modes of the large/noncubic workloads: wavevector k
    (integer, 0 < |k| <= nx/4), amplitude in [0.5, 1.5), phase in [0, 2 pi)."""
    nx = grid[0]
    rng = np.random.default_rng(seed)
    kmax = nx / 4
    out = []
    for _ in range(count):
        while True:
            k = rng.integers(-int(kmax), int(kmax) + 1, size=3)
            if 0 < np.sqrt((k ** 2).sum()) <= kmax:
                break
        amp = rng.uniform(0.5, 1.5)
        ph = rng.uniform(0, 2 * np.pi)
        out.append((tuple(int(v) for v in k), float(amp), float(ph)))
    return out


def make_input(torch, grid, seed, device, kind):
    """Seeded synthetic field on the device, (nz, ny, nx) float64: U[-1,1)
    ("uniform"), or the sum of modes_list's cosines plus N(0, 1e-3) noise."""
    nx, ny, nz = grid
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    if kind == "uniform":
        return torch.rand((nz, ny, nx), generator=g, device=device, dtype=torch.float64) * 2 - 1
    if kind == "cheby":
        return make_cheby_input(torch, grid, seed, device)
    x = torch.arange(nx, device=device, dtype=torch.float64) / nx
    y = torch.arange(ny, device=device, dtype=torch.float64) / ny
    z = torch.arange(nz, device=device, dtype=torch.float64) / nz
    f = torch.randn((nz, ny, nx), generator=g, device=device, dtype=torch.float64) * 1e-3
    for k, amp, ph in modes_list(grid, seed):
        # cos(2 pi (kx x + ky y + kz z) + ph), built separably
        ax = torch.exp(1j * (2 * np.pi * k[0] * x + ph))
        ay = torch.exp(1j * 2 * np.pi * k[1] * y)
        az = torch.exp(1j * 2 * np.pi * k[2] * z)
        for zi in range(0, nz, 64):  # chunk to bound temporaries
            blk = az[zi:zi + 64, None, None] * ay[None, :, None] * ax[None, None, :]
            f[zi:zi + 64] += amp * blk.real
    return f


def expected_modes(grid, modes):
    """Analytic forward (unnormalised, e^{-i}) spectrum of the modes field at
    the kept half (kx >= 0): amp N/2 e^{i ph} at k and amp N/2 e^{-i ph} at -k,
    each stored at its kx >= 0 representative.  {(iz, iy, ix): complex}."""
    nx, ny, nz = grid
    half = nx * ny * nz / 2.0
    want = {}
    for k, amp, ph in modes:
        for sgn in (1, -1):
            kx, ky, kz = (sgn * v for v in k)
            if kx < 0:
                continue
            idx = (kz % nz, ky % ny, kx)
            want[idx] = want.get(idx, 0) + amp * half * np.exp(1j * sgn * ph)
    return want


def make_cheby_input(torch, grid, seed, device):
    """The Chebyshev workload's field: z on the Gauss-Lobatto points
    cos(pi (k-1)/(nz-1)), f = sum of 16 seeded sin(2 pi a x) cos(2 pi b y)
    T_m(z) with a, b <= 64, m <= 128, plus U[-1e-6, 1e-6) noise."""
    import math
    nx, ny, nz = grid
    rng = np.random.default_rng(seed)
    xs = torch.arange(nx, device=device, dtype=torch.float64) / nx
    ys = torch.arange(ny, device=device, dtype=torch.float64) / ny
    zs = torch.cos(math.pi * torch.arange(nz, device=device, dtype=torch.float64) / (nz - 1))
    f = torch.zeros((nz, ny, nx), dtype=torch.float64, device=device)
    for _ in range(16):
        a, b, m = int(rng.integers(0, 65)), int(rng.integers(0, 65)), int(rng.integers(0, 129))
        tz = torch.cos(m * torch.arccos(zs.clamp(-1, 1)))  # T_m on the Lobatto points
        f += (torch.sin(2 * math.pi * a * xs)[None, None, :] * torch.cos(2 * math.pi * b * ys)[None, :, None]
              * tz[:, None, None])
    g = torch.Generator(device=device)
    g.manual_seed(seed + 1)
    f += 1e-6 * (torch.rand(f.shape, generator=g, device=device, dtype=torch.float64) * 2 - 1)
    return f


# ----------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                           "--format=csv,noheader,nounits", "-lms", "100"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        return False

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ------------------------------------------------------------ our arm
def bytes_model(grid, esize_real):
    """3-pass model per direction: X pass R + C, Y pass 2C, Z pass 2C."""
    nx, ny, nz = grid
    r = nx * ny * nz * esize_real
    c = (nx // 2 + 1) * ny * nz * 2 * esize_real
    return {"x": r + c, "y": 2 * c, "z": 2 * c, "dir": r + 5 * c, "rt": 2 * (r + 5 * c), "R": r, "C": c}


def time_device(torch, plan, x, b, r, ops, steps, warmup, stream):
    """Device-resident round trips, CUDA events on the plan's stream."""
    for _ in range(warmup):
        plan.ftran_r2c(x, b, op=ops[0], stream=stream)
        plan.btran_c2r(b, r, op=ops[1], stream=stream)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    plan.reset_timers()
    launches0 = plan.launches
    ev0.record(stream)
    for _ in range(steps):
        plan.ftran_r2c(x, b, op=ops[0], stream=stream)
        plan.btran_c2r(b, r, op=ops[1], stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    return ms, plan.launches - launches0


# ------------------------------------------------------------ replicas
def replica_env():
    """(world, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(torch, dist, value: float, device) -> float:
    """The slowest rank's time: every rank runs a full replica, so the job's
    time is the maximum over ranks (no data-path collective)."""
    if dist is None:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_gpts(world: int, points_per_replica: int, ms: float) -> float:
    """Whole-job throughput: the points of all replicas over the max time."""
    return world * points_per_replica / (ms * 1e-3) / 1e9


def rt_norm(grid, ops):
    """Round-trip normalisation: N for FFTs, nx ny 2 (nz - 1) with DCT-I on z
    (unnormalised REDFT00 twice) and nx ny 2 (nz + 1) with DST-I."""
    nx, ny, nz = grid
    z = ops[0][2]
    if z == "c":
        return nx * ny * 2 * (nz - 1)
    if z == "s":
        return nx * ny * 2 * (nz + 1)
    if z in "n0":
        return nx * ny
    return nx * ny * nz


def gpu_linf(a, w) -> float:
    return float((a - w).abs().max() / w.abs().max())


def gpu_rel_l2(torch, a, w) -> float:
    return float(torch.linalg.vector_norm(a - w) / torch.linalg.vector_norm(w))


def accuracy(torch, grid, ops, kind, x, plan64, plan32, stream, lz=None, seed=None):
    """Outputs on the full grid against the CPU oracle (numpy/scipy FP64
    restatement of the reference path, all host cores), outside any timed
    region: forward and backward of the F64 path (normalised L-inf, bound
    1e-12), of the F32 path (relative L2, bound 1e-6), the round trip under
    the samples' rule, the analytic spectrum of the modes field, and
    p3dfft_cheby for the Chebyshev workload."""
    from oracle import p3dfft_oracle as orc
    orc.WORKERS = os.cpu_count() or 1
    t0 = time.time()
    nx, ny, nz = grid
    n = nx * ny * nz
    dev = x.device
    ref = orc.OraclePlan(nx, ny, nz)
    a = x.cpu().numpy()
    wb_np = ref.ftran_r2c(a, ops[0])
    want_b = torch.from_numpy(wb_np).to(dev)
    b64 = plan64.ftran_r2c(x, op=ops[0], stream=stream)
    torch.cuda.synchronize()
    out = {"f64_forward_normalised_linf_vs_oracle": gpu_linf(b64, want_b)}
    if kind == "modes":
        want = expected_modes(grid, modes_list(grid, seed))
        idx = torch.tensor(list(want.keys()), device=dev)
        got = b64[idx[:, 0], idx[:, 1], idx[:, 2]]
        w = torch.tensor(list(want.values()), dtype=torch.complex128, device=dev)
        # the N(0, 1e-3) noise adds ~1e-3 sqrt(N) per mode against amplitudes of ~N/2
        out["f64_modes_max_rel_err"] = float(((got - w).abs() / w.abs()).max())
        out["modes_checked"] = len(want)
    r64 = plan64.btran_c2r(b64, op=ops[1], stream=stream)
    want_r = torch.from_numpy(ref.btran_c2r(wb_np, ops[1])).to(dev)
    torch.cuda.synchronize()
    out["f64_backward_normalised_linf_vs_oracle"] = gpu_linf(r64, want_r)
    rt = float((r64.div_(rt_norm(grid, ops)) - x).abs().max())
    out["f64_roundtrip_max_abs"] = rt
    out["f64_roundtrip_normalised_linf"] = rt / float(x.abs().max())
    out["roundtrip_rule_f64"] = 1e-14 * n * 0.25
    del r64
    if lz is not None:
        c = plan64.cheby(x, lz, stream=stream)
        want_c = torch.from_numpy(ref.cheby(a, lz)).to(dev)
        torch.cuda.synchronize()
        out["f64_cheby_normalised_linf_vs_oracle"] = gpu_linf(c, want_c)
        del c, want_c
    del b64
    if plan32 is not None:
        b32 = plan32.ftran_r2c(x.float(), op=ops[0], stream=stream)
        torch.cuda.synchronize()
        out["f32_forward_rel_l2_vs_oracle"] = gpu_rel_l2(torch, b32.to(torch.complex128), want_b)
        r32 = plan32.btran_c2r(want_b.to(torch.complex64), op=ops[1], stream=stream)
        torch.cuda.synchronize()
        out["f32_backward_rel_l2_vs_oracle"] = gpu_rel_l2(torch, r32.double(), want_r)
        r32 = plan32.btran_c2r(b32, op=ops[1], stream=stream)
        torch.cuda.synchronize()
        rt32 = float((r32.double().div_(rt_norm(grid, ops)) - x).abs().max())
        out["f32_roundtrip_max_abs"] = rt32
        out["roundtrip_rule_f32"] = 1e-5 * n * 0.25
        del b32, r32
    out["oracle_threads"] = orc.WORKERS
    out["oracle_s"] = round(time.time() - t0, 1)
    del want_b, want_r, wb_np, a
    return out


def pass_times(timers, steps):
    """Per-pass milliseconds per round trip from a plan's timer slots."""
    slots = {"x_r2c": 4, "y_fwd": 6, "z_fwd": 7, "z_bwd": 8, "y_bwd": 9, "x_c2r": 11}
    return {k: round(timers[i] * 1e3 / steps, 4) for k, i in slots.items()}


def measure_config(torch, pg, name, args, dev, stream, seed, with_accuracy=True, clock=None):
    """One workload: FP64 and FP32 round trips timed with CUDA events on the
    plan's stream (the plan timers give the per-pass times; `clock`, a
    ClockSampler, runs around the timed loops), then the outputs against the
    oracle."""
    import contextlib
    clock = clock if clock is not None else contextlib.nullcontext()
    cfg = CONFIGS[name]
    grid, ops = cfg["grid"], cfg["ops"]
    nx, ny, nz = grid
    npts = nx * ny * nz
    x = make_input(torch, grid, seed, dev, cfg["input"])
    res = {"workload": cfg["workload"], "grid": list(grid), "ops": list(ops)}
    plan = pg.Plan(nx, ny, nz, precision=pg.F64, timers=True)
    plan.set_options(*MODES[args.mode])
    b = torch.empty(plan.complex_shape, dtype=torch.complex128, device=dev)
    r = torch.empty_like(x)
    plan32 = pg.Plan(nx, ny, nz, precision=pg.F32, timers=True)
    plan32.set_options(*MODES[args.mode])
    x32 = x.float()
    b32 = torch.empty(plan32.complex_shape, dtype=torch.complex64, device=dev)
    r32 = torch.empty_like(x32)
    with clock:
        ms64, launches = time_device(torch, plan, x, b, r, ops, args.steps, args.warmup, stream)
        ms32, _ = time_device(torch, plan32, x32, b32, r32, ops, args.steps, args.warmup, stream)
    timers = plan.timers()
    t32 = plan32.timers()
    del b, r, x32, b32, r32
    peak, _ = load_peaks()
    bm64, bm32 = bytes_model(grid, 8), bytes_model(grid, 4)
    res.update({
        "f64": {"value": round(npts / (ms64 * 1e-3) / 1e9, 3), "unit": UNIT, "ms_per_step": round(ms64, 4),
                "step_frac_of_measured_hbm": round(bm64["rt"] / (ms64 * 1e-3) / 1e9 / peak, 4)},
        "f32": {"value": round(npts / (ms32 * 1e-3) / 1e9, 3), "unit": UNIT, "ms_per_step": round(ms32, 4),
                "step_frac_of_measured_hbm": round(bm32["rt"] / (ms32 * 1e-3) / 1e9 / peak, 4),
                "speedup_vs_f64": round(ms64 / ms32, 3), "passes_ms": pass_times(t32, args.steps)},
    })
    if with_accuracy:
        res["error"] = accuracy(torch, grid, ops, cfg["input"], x, plan, plan32, stream,
                                lz=2.0 if name == "cheby" else None, seed=seed)
    plan.close()
    plan32.close()
    del x
    torch.cuda.empty_cache()
    return res, ms64, ms32, timers, launches


def run_ours(args):
    import torch
    import p3dfft_gb300 as pg

    world, rank, local = replica_env()
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    cfg = CONFIGS[args.config]
    grid = cfg["grid"]
    nx, ny, nz = grid
    ops = cfg["ops"]
    npts = nx * ny * nz
    stream = torch.cuda.Stream(device=dev)
    peak, peak_kind = load_peaks()
    # every torch op and every plan call below runs on one stream
    ctx = torch.cuda.stream(stream)
    ctx.__enter__()
    seed = 1234 + rank

    # ---- FP64 (headline) and FP32 on the same grid, timed with clocks sampled
    if dist:
        dist.barrier()
    clk = ClockSampler(local)
    head, ms64, ms32, timers, launches = measure_config(torch, pg, args.config, args, dev, stream, seed,
                                                        with_accuracy=False, clock=clk)
    ms64 = max_over_ranks(torch, dist, ms64, dev)
    ms32 = max_over_ranks(torch, dist, ms32, dev)
    bm = bytes_model(grid, 8)
    pass_ms = {
        "x_r2c": timers[4] * 1e3 / args.steps, "y_fwd": timers[6] * 1e3 / args.steps,
        "z_fwd": timers[7] * 1e3 / args.steps, "z_bwd": timers[8] * 1e3 / args.steps,
        "y_bwd": timers[9] * 1e3 / args.steps, "x_c2r": timers[11] * 1e3 / args.steps,
    }
    pass_bytes = {"x_r2c": bm["x"], "y_fwd": bm["y"], "z_fwd": bm["z"], "z_bwd": bm["z"], "y_bwd": bm["y"],
                  "x_c2r": bm["x"]}
    # passes grouped by kernel; the dominant kernel is the one with the largest
    # total time per round trip (4 strided launches, 1 r2c, 1 c2r)
    groups = {"k_strided_pipe": ["y_fwd", "z_fwd", "z_bwd", "y_bwd"], "k_xr2c_pipe": ["x_r2c"],
              "k_xc2r_pipe": ["x_c2r"]}
    dom = max(groups, key=lambda k: sum(pass_ms[p] for p in groups[k]))
    nl = len(groups[dom])
    dom_ms = sum(pass_ms[p] for p in groups[dom]) / nl
    dom_bytes = sum(pass_bytes[p] for p in groups[dom]) / nl
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9 if dom_ms > 0 else None
    traffic = None
    if dom in TRAFFIC_PER_ALGO_BYTE:
        traffic = int(TRAFFIC_PER_ALGO_BYTE[dom] * dom_bytes)

    # ---- end to end through the drop-in C-ABI with pinned host buffers
    x = make_input(torch, grid, seed, dev, cfg["input"])
    e2e = None
    if not args.skip_e2e:
        e2e = run_e2e(torch, pg, grid, ops, x, max(1, args.steps // 2), dev)

    # ---- accuracy of the headline workload against the oracle (not timed)
    error = None
    if not args.skip_accuracy:
        plan = pg.Plan(nx, ny, nz, precision=pg.F64)
        plan32 = pg.Plan(nx, ny, nz, precision=pg.F32)
        error = accuracy(torch, grid, ops, cfg["input"], x, plan, plan32, stream,
                         lz=2.0 if args.config == "cheby" else None, seed=seed)
        plan.close()
        plan32.close()
    del x
    torch.cuda.empty_cache()

    # ---- the other configured workloads, each timed and checked against the oracle
    configs = {}
    if not args.skip_configs:
        for name in ("noncubic", "cheby", "small"):
            if name == args.config:
                continue
            configs[name] = measure_config(torch, pg, name, args, dev, stream, seed)[0]
    batched = serving = None
    if not args.skip_forms:
        batched = run_batched(torch, pg, dev, args.steps, args.warmup, npts / (ms64 * 1e-3) / 1e9)
        serving = run_serving(torch, pg, args.serve_requests, npts / (ms64 * 1e-3) / 1e9)

    value = aggregate_gpts(world, npts, ms64)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms64, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": cfg["workload"], "grid": list(grid), "ops": list(ops), "precision": "f64",
                   "arithmetic": "binary64 I/O, double-float (2 x binary32) butterflies",
                   "l2": "inputs larger than L2 (8 GB per field), no flush needed",
                   "parallelism": f"replicas x{world}"},
        "error": error,
        "f32": {"value": round(aggregate_gpts(world, npts, ms32), 3), "unit": UNIT, "ms_per_step": round(ms32, 4),
                "speedup_vs_f64": round(ms64 / ms32, 3),
                "step_frac": round(bytes_model(grid, 4)["rt"] / (ms32 * 1e-3) / 1e9 / peak, 4),
                "passes_ms": head["f32"]["passes_ms"]},
        "passes_ms": {k: round(v, 4) for k, v in pass_ms.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "launches_per_step": nl,
                     "algorithmic_bytes_per_launch": int(dom_bytes),
                     "avg_launch_ms": round(dom_ms, 4),
                     "achieved": round(achieved, 1) if achieved else None,
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "traffic_source": "ncu DRAM read+write of the Y pass (1024x1024x32) and Z passes "
                                       "(1024x32x1024), 0.923 per algorithmic byte, scaled to this launch",
                     "step_bytes_model": bm["rt"],
                     "step_frac": round(bm["rt"] / (ms64 * 1e-3) / 1e9 / peak, 4)},
        "gpu_launches": launches,
        "kernel_mode": args.mode,
        "clocks": clk.summary(),
    }
    if e2e:
        line["e2e"] = e2e
    if configs:
        line["configs"] = configs
    if batched:
        line["batched"] = batched
    if serving:
        line["serving"] = serving
    ctx.__exit__(None, None, None)
    if rank == 0 and not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline(args)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


BATCH_SIDES = (48, 64, 96, 120, 128, 160, 192, 256)


def run_batched(torch, pg, dev, steps, warmup, plain_f64_gpts):
    """Batching form: 64 independent r2c+c2r round trips, each side drawn
    from BATCH_SIDES with a fixed seed, inputs U[-1,1), in one persistent
    launch replayed from a captured CUDA graph; per-shape radix/tile knobs and
    the queue window from the autotuner.  Also times the same 64 round trips
    issued one plan call after another (the plain API) for comparison."""
    from p3dfft_gb300 import autotune
    rng = np.random.default_rng(4)
    shapes = [tuple(int(v) for v in rng.choice(BATCH_SIDES, size=3)) for _ in range(64)]
    npts = sum(a * b * c for a, b, c in shapes)
    out = {"grids": 64, "sides": list(BATCH_SIDES), "points_per_step": npts, "seed": 4}
    results = {}
    t_tune = time.time()
    for prec, name in ((pg.F64, "f64"), (pg.F32, "f32")):
        rdt = torch.float64 if prec == pg.F64 else torch.float32
        plans = {}
        for sh in sorted(set(shapes)):
            t = autotune.tune_shape(sh, prec, reps=3, min_points=1 << 23, cands=autotune.candidates(prec)[:3])
            plans[sh] = pg.Plan(*sh, precision=prec, max_radix=t["max_radix"], max_lines=t["max_lines"])
        g = torch.Generator(device=dev)
        g.manual_seed(44)
        jobs = []
        for sh in shapes:
            nx, ny, nz = sh
            x = torch.rand((nz, ny, nx), generator=g, device=dev, dtype=torch.float64).mul_(2).sub_(1).to(rdt)
            jobs.append({"plan": plans[sh], "kind": pg.JOB_ROUNDTRIP, "in": x,
                         "out": torch.empty_like(x)})
        window, wtimes = autotune.tune_window(jobs, prec, windows=(1, 4, 16, 0), reps=3)
        b = pg.Batch(prec).set_jobs(jobs, window=window)
        b.capture()
        stream = torch.cuda.current_stream()
        for _ in range(warmup):
            b.replay(stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            b.replay(stream)
        e1.record(stream)
        b.check(stream)
        ms = e0.elapsed_time(e1) / steps
        info = b.info()
        # round-trip error of every grid (unnormalised transform: divide by N)
        worst = 0.0
        for j in jobs:
            p = j["plan"]
            r = j["out"].double() / (p.nx * p.ny * p.nz)
            xin = j["in"].double()
            worst = max(worst, float(torch.linalg.vector_norm(r - xin) / torch.linalg.vector_norm(xin)))
        # the same round trips through the plain per-plan API, one after another
        for p in plans.values():
            p.set_options(True, True)
        for _ in range(2):
            for j in jobs:
                j["plan"].btran_c2r(j["plan"].ftran_r2c(j["in"]), j["out"])
        e0.record(stream)
        for _ in range(max(1, steps // 2)):
            for j in jobs:
                j["plan"].btran_c2r(j["plan"].ftran_r2c(j["in"]), j["out"])
        e1.record(stream)
        torch.cuda.synchronize()
        ms_plain = e0.elapsed_time(e1) / max(1, steps // 2)
        results[name] = {"value": round(npts / (ms * 1e-3) / 1e9, 3), "unit": UNIT, "ms_per_step": round(ms, 4),
                         "window": window, "window_ms": {str(k): round(v, 4) for k, v in wtimes.items()},
                         "work_items": info["items"], "persistent_ctas": info["ctas"],
                         "kernel_launches_per_step": 1, "roundtrip_rel_l2_max": worst,
                         "plain_api_ms_per_step": round(ms_plain, 4),
                         "speedup_vs_plain_api": round(ms_plain / ms, 3)}
        b.close()
        for p in plans.values():
            p.close()
        del jobs
        torch.cuda.empty_cache()
    out.update(results)
    out["tuning_s"] = round(time.time() - t_tune, 1)
    if plain_f64_gpts:
        out["f32_vs_plain_f64_1024cubed"] = round(results["f32"]["value"] / plain_f64_gpts, 3)
    # the same 64 grids: FP32 batched form against FP64 batched and against
    # FP64 through the plain per-plan API
    out["f32_vs_f64_batched_same_grids"] = round(results["f32"]["value"] / results["f64"]["value"], 3)
    out["f32_vs_f64_plain_api_same_grids"] = round(results["f64"]["plain_api_ms_per_step"] /
                                                   results["f32"]["ms_per_step"], 3)
    return out


def run_serving(torch, pg, n_requests, plain_f64_gpts, slots=3):
    """Serving form: requests (forward : backward : spectrum = 4:4:2, cubic or
    box grids with sides log-uniform over the 2^a 3^b 5^c values in [32,512],
    10 % asking for FP64 accuracy) through the continuous-batching server with
    a 150 GB device-memory budget, in two runs: every request with its own
    host input and result (H2D and D2H inside its latency), and every request
    with its own device input (a view of a device arena; no host transfer).
    Each run measures its capacity first with a closed loop (600 requests
    queued at once); its timed stream then arrives as a Poisson process at
    70 % of that capacity."""
    from p3dfft_gb300 import serve
    srv = serve.Server(budget_bytes=150e9, slots=slots, max_jobs=64, window=4, keep_outputs=False,
                       launch_work=20e6, age_limit=0.008)

    def one(attach, seed_cap, seed_run):
        cap_reqs = serve.make_requests(min(600, n_requests), seed=seed_cap)
        reqs = serve.poisson_arrivals(serve.make_requests(n_requests, seed=seed_run), rate=1.0)
        attach(cap_reqs + reqs)
        t = time.time()
        for r in cap_reqs + reqs:  # plans (tables) resident before the clock starts
            srv.plan(r.shape, pg.F64 if r.tol < serve.F32_TOL else pg.F32)
        plan_s = time.time() - t
        srv.run(serve.make_requests(64, seed=51))  # warm-up
        t = time.perf_counter()
        srv.run(cap_reqs)
        cap_wall = time.perf_counter() - t
        capacity = len(cap_reqs) / cap_wall
        rate = 0.7 * capacity
        serve.poisson_arrivals(reqs, rate=rate, seed=6)
        launches0 = srv.launches
        t = time.perf_counter()
        srv.run(reqs)
        wall = time.perf_counter() - t
        out = serve.summarize(reqs, wall)
        out.update({"arrival_rate_req_s": round(rate, 1), "capacity_req_s": round(capacity, 1),
                    "capacity_gpts_s": round(sum(r.points for r in cap_reqs) / cap_wall / 1e9, 3),
                    "launches": srv.launches - launches0,
                    "mean_jobs_per_launch": round(float(np.mean(srv.batch_sizes[-(srv.launches - launches0):]
                                                                or [0])), 2),
                    "fallbacks": sum(1 for r in reqs if r.fallback), "plan_setup_s": round(plan_s, 1)})
        if plain_f64_gpts:
            out["capacity_vs_plain_f64_1024cubed"] = round(out["capacity_gpts_s"] / plain_f64_gpts, 3)
        return out

    # every request brings its own host input and takes its result back to the
    # host (views rotating through two 2 GiB page-locked arenas)
    out = one(lambda rs: serve.attach_host_data(rs, arena_bytes=2 << 30), 50, 5)
    out.update({"budget_gb": 150, "peak_in_flight_gb": round(srv.peak_in_flight / 1e9, 2), "slots": len(srv.slots),
                "plans_resident": len(srv.plans), "mix": "forward:backward:spectrum 4:4:2, 10% FP64",
                "data": "per request: H2D of its own input and D2H of its result on its launch's stream, "
                        "inside the latency",
                "schedule": "least estimated work first, launches bounded at 20M point-equivalents, "
                            "requests waiting 8 ms first"})
    # every request transforms its own device buffer (views rotating through
    # an 8 GiB device arena): the kernels' and the scheduler's share
    dev = one(lambda rs: serve.attach_device_data(rs, arena_bytes=8 << 30), 52, 7)
    dev["data"] = "per request: its own input buffer in device memory (no host transfer)"
    out["device_data"] = dev
    srv.close()
    return out


def run_e2e(torch, pg, grid, ops, x_dev, steps, dev):
    """Same metric through the reference-facing C-ABI (p3dfft_ftran_r2c /
    p3dfft_btran_c2r) with pinned host buffers: H2D and D2H inside the timing."""
    nx, ny, nz = grid
    host_in = torch.empty((nz, ny, nx), dtype=torch.float64, pin_memory=True)
    host_in.copy_(x_dev.cpu())
    host_c = torch.empty((nz, ny, nx // 2 + 1), dtype=torch.complex128, pin_memory=True)
    host_out = torch.empty((nz, ny, nx), dtype=torch.float64, pin_memory=True)
    pg.p3dfft_setup((1, 1), nx, ny, nz, 0, nx, ny, nz, True)
    try:
        pg.p3dfft_ftran_r2c(host_in, host_c, ops[0])
        pg.p3dfft_btran_c2r(host_c, host_out, ops[1])
        tf = tb = 0.0
        t0 = time.perf_counter()
        for _ in range(steps):
            t1 = time.perf_counter()
            pg.p3dfft_ftran_r2c(host_in, host_c, ops[0])
            t2 = time.perf_counter()
            pg.p3dfft_btran_c2r(host_c, host_out, ops[1])
            tf += t2 - t1
            tb += time.perf_counter() - t2
        dt = (time.perf_counter() - t0) / steps
    finally:
        pg.p3dfft_clean()
    r_bytes = nx * ny * nz * 8
    c_bytes = (nx // 2 + 1) * ny * nz * 16
    # host-link bandwidth seen by pinned copies of the same arrays (1 GiB each way)
    link = {}
    n = min(host_in.numel(), 1 << 27)
    dbuf = torch.empty(n, dtype=torch.float64, device=dev)
    hflat = host_in.view(-1)[:n]
    for name, fn in (("h2d", lambda: dbuf.copy_(hflat, non_blocking=True)),
                     ("d2h", lambda: hflat.copy_(dbuf, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        link[name] = round(n * 8 / (time.perf_counter() - t) / 1e9, 1)
    del dbuf
    return {"value": round(nx * ny * nz / dt / 1e9, 3), "unit": UNIT, "ms_per_step": round(dt * 1e3, 3),
            "ftran_ms": round(tf / steps * 1e3, 3), "btran_ms": round(tb / steps * 1e3, 3),
            "h2d_bytes_per_step": r_bytes + c_bytes, "d2h_bytes_per_step": c_bytes + r_bytes,
            "path": "libp3dfft.so p3dfft_ftran_r2c + p3dfft_btran_c2r, pinned host arrays: the real arrays "
                    "read/written in place by the X passes over the host link, the complex arrays copied in "
                    "row blocks overlapped with the Z pass",
            "host_link_gbs": link}


# ------------------------------------------------------------ CPU arms
def cpu_round_trips(grid, ops, seconds, max_steps=None, warmup=1):
    """Round trips of the whole grid through the oracle port on every host
    core (U[-1,1) input: the FFT's time does not depend on the values)."""
    from oracle import p3dfft_oracle as orc
    orc.WORKERS = os.cpu_count() or 1
    nx, ny, nz = grid
    a = np.random.default_rng(7).uniform(-1, 1, size=(nz, ny, nx))
    p = orc.OraclePlan(nx, ny, nz)
    for _ in range(warmup):  # plans, page faults
        p.btran_c2r(p.ftran_r2c(a, ops[0]), ops[1])
    n = 0
    t0 = time.perf_counter()
    while True:
        b = p.ftran_r2c(a, ops[0])
        p.btran_c2r(b, ops[1])
        del b
        n += 1
        el = time.perf_counter() - t0
        if (max_steps and n >= max_steps) or (not max_steps and el >= seconds):
            break
    return n, el, orc.WORKERS


def cpu_baseline(args):
    grid = CONFIGS[args.config]["grid"]
    ops = CONFIGS[args.config]["ops"]
    n, el, cores = cpu_round_trips(grid, ops, seconds=args.cpu_seconds)
    pts = grid[0] * grid[1] * grid[2]
    return {"value": round(pts * n / el / 1e9, 4), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} FP64 r2c+c2r round trips of the whole {grid[0]}x{grid[1]}x{grid[2]} grid after one "
                      f"untimed (oracle: numpy/scipy pocketfft restatement of the reference path, scipy.fft "
                      f"workers={cores}); the FFTW+MPI reference does not build here (no Fortran/MPI/FFTW)"}


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    grid = CONFIGS[args.config]["grid"]
    ops = CONFIGS[args.config]["ops"]
    n, el, cores = cpu_round_trips(grid, ops, seconds=0, max_steps=args.steps, warmup=args.warmup)
    pts = grid[0] * grid[1] * grid[2]
    value = pts * n / el / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el / n * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": CONFIGS[args.config]["workload"], "grid": list(grid), "sample_grid": list(grid),
                   "ops": list(ops)},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"each step one FP64 round trip of the whole {grid[0]}x{grid[1]}x{grid[2]} "
                                   f"grid through the oracle port (scipy.fft, {cores} threads; U[-1,1) input, "
                                   f"the FFT's time does not depend on the values); the FFTW+MPI reference does "
                                   f"not build here"},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="large", choices=sorted(CONFIGS))
    ap.add_argument("--mode", default="pipe_tma", choices=sorted(MODES),
                    help="kernel family: persistent pipelined with TMA or cp.async copies, or single-tile")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-forms", action="store_true", help="skip the batched and serving forms")
    ap.add_argument("--serve-requests", type=int, default=10000)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true", help="skip the oracle comparisons of the headline grid")
    ap.add_argument("--skip-configs", action="store_true", help="skip the other configured workloads")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
