"""Batch driver: round trips of many uneven grids in one persistent launch.

  python -m p3dfft_gb300.batchrun --grids 64 --precision f32 --steps 3
  python -m p3dfft_gb300.batchrun --shape 128 128 128 --grids 16

Grids are drawn (seeded) from the sides 48..256 of the batched workload, or
all of one --shape; inputs U[-1,1).  Prints the time per graph replay (CUDA
events) and the points per second.  Used for quick checks and as the
workload of the batch kernel's ncu captures.
"""
from __future__ import annotations

import argparse
import json

SIDES = (48, 64, 96, 120, 128, 160, 192, 256)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--grids", type=int, default=64)
    ap.add_argument("--shape", type=int, nargs=3, default=None)
    ap.add_argument("--precision", choices=["f64", "f32"], default="f32")
    ap.add_argument("--window", type=int, default=0)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--seed", type=int, default=4)
    args = ap.parse_args(argv)

    import numpy as np
    import torch

    import p3dfft_gb300 as pg

    prec = pg.F64 if args.precision == "f64" else pg.F32
    rdt = torch.float64 if prec == pg.F64 else torch.float32
    rng = np.random.default_rng(args.seed)
    if args.shape:
        shapes = [tuple(args.shape)] * args.grids
    else:
        shapes = [tuple(int(v) for v in rng.choice(SIDES, size=3)) for _ in range(args.grids)]
    plans = {sh: pg.Plan(*sh, precision=prec) for sh in set(shapes)}
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed)
    jobs = []
    for sh in shapes:
        nx, ny, nz = sh
        x = torch.rand((nz, ny, nx), generator=g, device="cuda", dtype=rdt).mul_(2).sub_(1)
        jobs.append({"plan": plans[sh], "kind": pg.JOB_ROUNDTRIP, "in": x, "out": torch.empty_like(x)})
    b = pg.Batch(prec).set_jobs(jobs, window=args.window)
    b.capture()
    stream = torch.cuda.current_stream()
    b.replay(stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.replay(stream)
    e1.record(stream)
    b.check(stream)
    ms = e0.elapsed_time(e1) / args.steps
    npts = sum(a * c * d for a, c, d in shapes)
    print(json.dumps({"grids": len(shapes), "precision": args.precision, "window": args.window,
                      "ms_per_step": round(ms, 4), "gpts_per_s": round(npts / (ms * 1e-3) / 1e9, 3),
                      **b.info()}))
    b.close()


if __name__ == "__main__":
    main()
