"""Round-trip driver: forward r2c then backward c2r of one seeded grid.

  python -m p3dfft_gb300.roundtrip --grid 1024 1024 32 --precision f64 --steps 2

Prints the per-step time (CUDA events), the per-pass timers and the
normalised round-trip error.  Used for quick checks and as the workload of
the ncu captures summarised under profiles/.
"""
from __future__ import annotations

import argparse
import json

MODES = {"pipe_tma": (True, True), "pipe_cpasync": (True, False), "single_tile": (False, False)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, nargs=3, default=[128, 128, 128], metavar=("NX", "NY", "NZ"))
    ap.add_argument("--precision", choices=["f64", "f32"], default="f64")
    ap.add_argument("--ops", nargs=2, default=["fft", "tff"])
    ap.add_argument("--mode", choices=sorted(MODES), default="pipe_tma")
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--max-radix", type=int, default=0, help="largest power-of-two radix (plan tuning knob)")
    ap.add_argument("--max-lines", type=int, default=0, help="most lines per tile (plan tuning knob)")
    args = ap.parse_args(argv)

    import torch

    import p3dfft_gb300 as pg

    nx, ny, nz = args.grid
    f64 = args.precision == "f64"
    plan = pg.Plan(nx, ny, nz, precision=pg.F64 if f64 else pg.F32, timers=True, max_radix=args.max_radix,
                   max_lines=args.max_lines)
    plan.set_options(*MODES[args.mode])
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed)
    x = torch.rand((nz, ny, nx), generator=g, device="cuda", dtype=torch.float64 if f64 else torch.float32) * 2 - 1
    b = plan.ftran_r2c(x, op=args.ops[0])
    r = plan.btran_c2r(b, op=args.ops[1])
    torch.cuda.synchronize()
    plan.reset_timers()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        plan.ftran_r2c(x, b, op=args.ops[0])
        plan.btran_c2r(b, r, op=args.ops[1])
    e1.record()
    torch.cuda.synchronize()
    plan.check()
    ms = e0.elapsed_time(e1) / args.steps
    t = plan.timers()
    scale = 1.0 / (nx * ny * nz)
    if args.ops == ["fft", "tff"]:
        err = float((r * scale - x).abs().max() / x.abs().max())
    else:
        err = None
    print(json.dumps({"grid": [nx, ny, nz], "precision": args.precision, "mode": args.mode,
                      "max_radix": args.max_radix, "max_lines": args.max_lines,
                      "ms_per_round_trip": round(ms, 4),
                      "passes_ms": {name: round(t[i] * 1e3 / args.steps, 4) for name, i in
                                    (("x_r2c", 4), ("y_fwd", 6), ("z_fwd", 7), ("z_bwd", 8), ("y_bwd", 9),
                                     ("x_c2r", 11))},
                      "roundtrip_normalised_linf": err, "launches": plan.launches}))
    plan.close()


if __name__ == "__main__":
    main()
