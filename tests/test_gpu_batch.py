"""Batches of uneven transforms in one persistent launch (p3g_batch_*).

Every job of a batch must give the same result as the same transform run
alone through the plan's single-tile kernels (bit for bit: same codelets,
same twiddles, same stage plans), whatever the other jobs, the queue window
or the launch route (direct launch, captured CUDA graph); and the oracle
tolerances hold (F64 normalised L-inf <= 1e-12, F32 relative L2 <= 1e-6).
"""
import numpy as np
import pytest

from oracle import p3dfft_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300  # noqa: F401
    return torch


SHAPES = [(48, 64, 96), (120, 64, 48), (32, 30, 20), (15, 9, 7), (64, 64, 64), (96, 48, 160), (16, 12, 10)]


def _rdt(torch, prec):
    import p3dfft_gb300 as pg
    return (torch.float64, torch.complex128) if prec == pg.F64 else (torch.float32, torch.complex64)


def _alone(torch, plan, kind, x):
    """The same job through the plan's single-tile kernels."""
    import p3dfft_gb300 as pg
    plan.set_options(False, False)
    if kind == pg.JOB_FORWARD:
        return plan.ftran_r2c(x)
    if kind == pg.JOB_BACKWARD:
        return plan.btran_c2r(x)
    return plan.btran_c2r(plan.ftran_r2c(x))


def _make_jobs(torch, shapes, kinds, prec, seed=0, **plan_kw):
    import p3dfft_gb300 as pg
    rdt, cdt = _rdt(torch, prec)
    rng = np.random.default_rng(seed)
    jobs = []
    for (nx, ny, nz), kind in zip(shapes, kinds):
        plan = pg.Plan(nx, ny, nz, precision=prec, **plan_kw)
        if kind == pg.JOB_BACKWARD:
            # a valid r2c spectrum: the forward transform of a real field
            x0 = torch.from_numpy(rng.uniform(-1, 1, (nz, ny, nx))).to("cuda", rdt)
            inp = plan.ftran_r2c(x0)
            out = torch.empty((nz, ny, nx), dtype=rdt, device="cuda")
        else:
            inp = torch.from_numpy(rng.uniform(-1, 1, (nz, ny, nx))).to("cuda", rdt)
            shape = plan.complex_shape if kind == pg.JOB_FORWARD else (nz, ny, nx)
            out = torch.empty(shape, dtype=cdt if kind == pg.JOB_FORWARD else rdt, device="cuda")
        jobs.append({"plan": plan, "kind": kind, "in": inp, "out": out})
    return jobs


@pytest.mark.parametrize("window", [0, 1, 3])
def test_batch_roundtrip_matches_alone_f64(torch_cuda, window):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    jobs = _make_jobs(torch, SHAPES, [pg.JOB_ROUNDTRIP] * len(SHAPES), pg.F64, seed=1)
    b = pg.Batch(pg.F64).set_jobs(jobs, window=window)
    b.launch()
    b.check()
    for j in jobs:
        want = _alone(torch, j["plan"], j["kind"], j["in"])
        torch.cuda.synchronize()
        assert torch.equal(j["out"], want)
        p = j["plan"]
        a = j["in"].cpu().numpy()
        ref = orc.OraclePlan(p.nx, p.ny, p.nz)
        assert orc.normalised_linf(j["out"].cpu().numpy(), ref.btran_c2r(ref.ftran_r2c(a))) <= 1e-12
    b.close()


def test_batch_mixed_kinds_and_graph_replay(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    kinds = [pg.JOB_FORWARD, pg.JOB_BACKWARD, pg.JOB_ROUNDTRIP, pg.JOB_FORWARD, pg.JOB_BACKWARD,
             pg.JOB_ROUNDTRIP, pg.JOB_FORWARD]
    jobs = _make_jobs(torch, SHAPES, kinds, pg.F64, seed=2)
    b = pg.Batch(pg.F64).set_jobs(jobs, window=2)
    b.capture()
    for _ in range(2):
        for j in jobs:
            j["out"].zero_()
        b.replay()
        b.check()
        for j in jobs:
            want = _alone(torch, j["plan"], j["kind"], j["in"])
            torch.cuda.synchronize()
            assert torch.equal(j["out"], want), (j["plan"].nx, j["plan"].ny, j["plan"].nz, j["kind"])
    assert b.info()["launches"] == 2
    b.close()


def test_batch_job_same_alone_and_in_mix(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    jobs = _make_jobs(torch, SHAPES, [pg.JOB_ROUNDTRIP] * len(SHAPES), pg.F64, seed=3)
    mix = pg.Batch(pg.F64).set_jobs(jobs)
    mix.launch()
    mix.check()
    together = [j["out"].clone() for j in jobs]
    for j, t in zip(jobs, together):
        one = pg.Batch(pg.F64).set_jobs([j])
        j["out"].zero_()
        one.launch()
        one.check()
        assert torch.equal(j["out"], t)
        one.close()
    mix.close()


def test_batch_f32(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    shapes = SHAPES[:5]
    jobs = _make_jobs(torch, shapes, [pg.JOB_FORWARD] * len(shapes), pg.F32, seed=4)
    b = pg.Batch(pg.F32).set_jobs(jobs)
    b.launch()
    b.check()
    for j in jobs:
        want = _alone(torch, j["plan"], j["kind"], j["in"])
        torch.cuda.synchronize()
        assert torch.equal(j["out"], want)
        p = j["plan"]
        ref = orc.OraclePlan(p.nx, p.ny, p.nz).ftran_r2c(j["in"].double().cpu().numpy())
        assert orc.relative_l2(j["out"].cpu().numpy().astype(np.complex128), ref) <= 1e-6
    b.close()


def test_batch_spectrum_jobs(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    shapes = [(32, 30, 20), (48, 64, 96), (15, 9, 7)]
    rng = np.random.default_rng(5)
    jobs = []
    for nx, ny, nz in shapes:
        plan = pg.Plan(nx, ny, nz, precision=pg.F64)
        x = torch.from_numpy(rng.uniform(-1, 1, (nz, ny, nx))).cuda()
        kmax = int(np.sqrt(nx * nx + ny * ny + nz * nz) * 0.5 + 0.5)
        e = torch.empty(kmax + 1, dtype=torch.float64, device="cuda")
        jobs.append({"plan": plan, "kind": pg.JOB_SPECTRUM, "in": x, "out": e, "scale": 1.0 / (nx * ny * nz),
                     "flags": pg.SPEC_HERMITIAN})
    b = pg.Batch(pg.F64).set_jobs(jobs)
    b.launch()
    b.check()
    for j in jobs:
        p = j["plan"]
        bh = p.ftran_r2c(j["in"]).cpu().numpy() / (p.nx * p.ny * p.nz)
        want = orc.shell_spectrum(bh, p.nx, p.ny, p.nz, k2_weight=False, hermitian=True)
        assert orc.normalised_linf(j["out"].cpu().numpy(), want) <= 1e-12
        # Parseval on the field itself
        a = j["in"].cpu().numpy()
        assert abs(j["out"].sum().item() - np.sum(a * a) / a.size) <= 1e-12 * np.sum(a * a) / a.size
    b.close()


def test_batch_pruned_stride1_and_tuned_plans(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    plans = [pg.Plan(64, 48, 40, 40, 30, 24, precision=pg.F64),
             pg.Plan(32, 24, 20, precision=pg.F64, layout=pg.LAYOUT_STRIDE1),
             pg.Plan(128, 64, 32, precision=pg.F64, max_radix=4, max_lines=8),
             pg.Plan(96, 60, 40, precision=pg.F64, max_radix=2)]
    rng = np.random.default_rng(6)
    jobs = []
    for p in plans:
        x = torch.from_numpy(rng.uniform(-1, 1, (p.nz, p.ny, p.nx))).cuda()
        out = torch.empty(p.complex_shape, dtype=torch.complex128, device="cuda")
        jobs.append({"plan": p, "kind": pg.JOB_FORWARD, "in": x, "out": out})
    b = pg.Batch(pg.F64).set_jobs(jobs, window=1)
    b.launch()
    b.check()
    for j in jobs:
        p = j["plan"]
        ref = orc.OraclePlan(p.nx, p.ny, p.nz, p.nxc, p.nyc, p.nzc, stride1=p.layout == pg.LAYOUT_STRIDE1)
        assert orc.normalised_linf(j["out"].cpu().numpy(), ref.ftran_r2c(j["in"].cpu().numpy())) <= 1e-12
    b.close()


def test_batch_many_small_grids(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    rng = np.random.default_rng(7)
    shapes = [tuple(int(v) for v in rng.choice([8, 12, 16, 20, 24, 30, 32], size=3)) for _ in range(40)]
    jobs = _make_jobs(torch, shapes, [pg.JOB_ROUNDTRIP] * len(shapes), pg.F64, seed=8)
    b = pg.Batch(pg.F64).set_jobs(jobs, window=8)
    b.launch()
    b.check()
    for j in jobs:
        want = _alone(torch, j["plan"], j["kind"], j["in"])
        torch.cuda.synchronize()
        assert torch.equal(j["out"], want)
    b.close()


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_batch_long_lines_use_large_ctas(torch_cuda, prec):
    # batches of lines up to 2048 points run 128-thread CTAs; a 4096-point
    # line needs the 256-thread tile, and the results stay the plain API's
    import p3dfft_gb300 as pg
    torch = torch_cuda
    precision = pg.F64 if prec == "f64" else pg.F32
    small = _make_jobs(torch, [(64, 48, 40), (2048, 4, 6)], [pg.JOB_ROUNDTRIP] * 2, precision, seed=9)
    b = pg.Batch(precision).set_jobs(small)
    assert b.info()["threads"] == 128
    b.close()
    jobs = _make_jobs(torch, [(4096, 6, 4), (64, 48, 40), (8, 4096, 2)], [pg.JOB_ROUNDTRIP] * 3, precision, seed=10)
    b = pg.Batch(precision).set_jobs(jobs)
    assert b.info()["threads"] == 256
    b.launch()
    b.check()
    for j in jobs:
        want = _alone(torch, j["plan"], j["kind"], j["in"])
        torch.cuda.synchronize()
        assert torch.equal(j["out"], want)
    b.close()


def test_batch_new_jobs_launched_on_another_stream(torch_cuda):
    # set_jobs right after a launch, and the next launch on another stream:
    # the new table reaches the device only after the running launch, whose
    # results stay those of its own jobs
    import p3dfft_gb300 as pg
    torch = torch_cuda
    a = _make_jobs(torch, SHAPES[:3], [pg.JOB_ROUNDTRIP] * 3, pg.F32, seed=11)
    c = _make_jobs(torch, SHAPES[3:6], [pg.JOB_FORWARD] * 3, pg.F32, seed=12)
    for j in a + c:  # work buffers that outlive every launch
        j["work"] = torch.empty(j["plan"].work_bytes(j["kind"]), dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    s1.wait_stream(torch.cuda.current_stream())
    s2.wait_stream(torch.cuda.current_stream())
    b = pg.Batch(pg.F32).set_jobs(a)
    for _ in range(3):
        b.set_jobs(a)
        b.launch(s1)
        b.set_jobs(c)
        b.launch(s2)
        b.check(s2)
        b.check(s1)
    torch.cuda.synchronize()
    for j in a + c:
        want = _alone(torch, j["plan"], j["kind"], j["in"])
        torch.cuda.synchronize()
        assert torch.equal(j["out"], want)
    b.close()


def test_batch_rejects_mixed_precision(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    jobs = _make_jobs(torch, [(16, 16, 16)], [pg.JOB_FORWARD], pg.F32)
    b = pg.Batch(pg.F64)
    with pytest.raises(pg.P3DFFTError, match="precision"):
        b.set_jobs(jobs)
    b.close()


def test_autotuner_picks_and_caches(torch_cuda, tmp_path, monkeypatch):
    import json

    import p3dfft_gb300 as pg
    from p3dfft_gb300 import autotune
    torch = torch_cuda
    monkeypatch.setenv(autotune.CACHE_ENV, str(tmp_path / "tune.json"))
    best = autotune.tune_shape((48, 40, 30), pg.F64, reps=2)
    assert (best["max_radix"], best["max_lines"]) in autotune.candidates(pg.F64)
    assert len(best["tried"]) >= 2 and best["ms"] > 0
    cached = json.loads((tmp_path / "tune.json").read_text())
    assert any(k.endswith("|f64|48x40x30") for k in cached)
    assert autotune.tune_shape((48, 40, 30), pg.F64) == best  # served from the cache
    plan = autotune.tuned_plan((48, 40, 30), pg.F64)
    assert plan.tuning == (best["max_radix"], best["max_lines"])
    jobs = _make_jobs(torch, SHAPES[:4], [pg.JOB_ROUNDTRIP] * 4, pg.F64, seed=9)
    w, times = autotune.tune_window(jobs, pg.F64, reps=2)
    assert w in times and all(t > 0 for t in times.values())


def test_batch_dependency_wait_times_out_and_context_survives(torch_cuda):
    # a dependency that can never complete: every wait on it runs out after
    # its poll limit (~4 s), the launch ends, the status reports the time-out,
    # and the next batch on the same context works
    import time

    import p3dfft_gb300 as pg
    torch = torch_cuda
    jobs = _make_jobs(torch, SHAPES[:2], [pg.JOB_ROUNDTRIP] * 2, pg.F64, seed=10)
    b = pg.Batch(pg.F64).set_jobs(jobs)
    b.block_pass(0)  # the X pass of job 0: its Y pass waits forever
    t = time.perf_counter()
    b.launch()
    with pytest.raises(pg.P3DFFTError, match="timed out"):
        b.check()
    assert time.perf_counter() - t < 60
    b.set_jobs(jobs)
    b.launch()
    b.check()
    for j in jobs:
        want = _alone(torch, j["plan"], j["kind"], j["in"])
        torch.cuda.synchronize()
        assert torch.equal(j["out"], want)
    b.close()
