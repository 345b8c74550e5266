"""Binary64 range of the F64 path (double-float butterflies with binary32's
exponent range) on the GPU.

The reference computes in binary64 throughout (build/fft_exec.F90:495-540,
p3dfft_type = KIND(1.0d0) at build/module.F90:92), so fields of any
magnitude binary64 holds transform correctly.  Here every F64 transform
scales its input by an exact 2^-k and its output by 2^k:

* the drop-in library picks k itself (re-running a call whose input was out
  of the window; in-place calls measure the input on the device first) and
  matches the oracle at every scale;
* the explicit API with P3G_RANGE_AUTO matches the oracle at every scale, in
  every kernel family (pipelined TMA, pipelined cp.async, single-tile);
* the explicit API with the default fixed bias reports P3G_E_RANGE (never a
  silent inf or zero) and, at the bias it reports, matches the oracle.

Tolerance: normalised L-inf 1e-12 against the oracle run on the same scaled
data (the scaling is exact, so the error is the unscaled transform's).
"""
import numpy as np
import pytest

from oracle import p3dfft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-12
SCALES = [2.0 ** 600, 2.0 ** -600, 1e300, 1e-300, 1e30, 1e-30, 1.0]
MODES = {"pipe_tma": (True, True), "pipe_cpasync": (True, False), "single_tile": (False, False)}


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300  # noqa: F401
    return torch


def _field(shape, seed, scale):
    return np.random.default_rng(seed).uniform(-1, 1, size=shape) * scale


def _spectrum(shape, seed, scale):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * scale


@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("scale", SCALES)
def test_auto_bias_matches_oracle_at_any_scale(torch_cuda, mode, scale):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = 48, 40, 36
    plan = pg.Plan(nx, ny, nz, precision=pg.F64)
    plan.set_options(*MODES[mode])
    plan.set_range(pg.RANGE_AUTO)
    ref = orc.OraclePlan(nx, ny, nz)
    a = _field((nz, ny, nx), 1, scale)
    b = plan.ftran_r2c(torch.from_numpy(a).cuda())
    want = ref.ftran_r2c(a, "fft")
    c = _spectrum(want.shape, 2, scale)
    r = plan.btran_c2r(torch.from_numpy(c).cuda())
    plan.check()
    assert orc.normalised_linf(b.cpu().numpy(), want) <= TOL
    assert orc.normalised_linf(r.cpu().numpy(), ref.btran_c2r(c, "tff")) <= TOL
    plan.close()


@pytest.mark.parametrize("case", [((32, 24, 17), "ffc", "cff", False), ((24, 20, 18), "ffs", "sff", False),
                                  ((40, 24, 30), "fft", "tff", True), ((30, 18, 17, 30, 9, 10), "fft", "tff", False)])
def test_auto_bias_z_ops_stride1_pruned(torch_cuda, case):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    args, opf, opb, stride1 = case
    nx, ny, nz = args[:3]
    plan = pg.Plan(*args, precision=pg.F64, layout=pg.LAYOUT_STRIDE1 if stride1 else pg.LAYOUT_XYZ)
    plan.set_range(pg.RANGE_AUTO)
    ref = orc.OraclePlan(*args, stride1=stride1)
    for scale in (2.0 ** 700, 2.0 ** -700):
        a = _field((nz, ny, nx), 3, scale)
        want = ref.ftran_r2c(a, opf)
        b = plan.ftran_r2c(torch.from_numpy(a).cuda(), op=opf)
        c = _spectrum(want.shape, 4, scale)
        r = plan.btran_c2r(torch.from_numpy(c).cuda(), op=opb)
        plan.check()
        assert orc.normalised_linf(b.cpu().numpy(), want) <= TOL
        assert orc.normalised_linf(r.cpu().numpy(), ref.btran_c2r(c, opb)) <= TOL
    plan.close()


def test_fixed_bias_reports_out_of_window_inputs(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = 32, 24, 20
    plan = pg.Plan(nx, ny, nz, precision=pg.F64)
    ref = orc.OraclePlan(nx, ny, nz)
    # inside the window: no report, no bias needed
    x = torch.from_numpy(_field((nz, ny, nx), 5, 1.0)).cuda()
    plan.ftran_r2c(x)
    assert plan.check_range()[:2] == (0, 0)
    for scale, emax in ((2.0 ** 600, 599), (2.0 ** -600, -601), (1e35, 116)):
        a = _field((nz, ny, nx), 6, scale)
        x = torch.from_numpy(a).cuda()
        plan.ftran_r2c(x)
        with pytest.raises(pg.P3DFFTError, match="exponent window"):
            plan.check()
        plan.ftran_r2c(x)
        rc, bias, e = plan.check_range()
        assert rc == pg.E_RANGE and e == emax and bias == emax
        plan.set_range(pg.RANGE_FIXED, bias)
        b = plan.ftran_r2c(x)
        plan.check()
        assert orc.normalised_linf(b.cpu().numpy(), ref.ftran_r2c(a, "fft")) <= TOL
        plan.set_range(pg.RANGE_FIXED, 0)
    # the backward input is checked the same way
    c = _spectrum((nz, ny, nx // 2 + 1), 7, 2.0 ** -900)
    plan.btran_c2r(torch.from_numpy(c).cuda())
    rc, bias, _ = plan.check_range()
    assert rc == pg.E_RANGE and bias < -800
    plan.close()


@pytest.mark.parametrize("scale", SCALES)
def test_dropin_matches_oracle_at_any_scale(torch_cuda, scale):
    import p3dfft_gb300 as pg
    nx, ny, nz = 32, 20, 18
    ref = orc.OraclePlan(nx, ny, nz)
    pg.p3dfft_setup((1, 1), nx, ny, nz)
    try:
        for rep in range(2):  # the second call starts at the bias the first needed
            a = _field((nz, ny, nx), 8 + rep, scale)
            b = np.zeros((nz, ny, nx // 2 + 1), np.complex128)
            pg.p3dfft_ftran_r2c(a, b, "fft")
            want = ref.ftran_r2c(a, "fft")
            assert orc.normalised_linf(b, want) <= TOL
            c = _spectrum(want.shape, 10 + rep, scale)
            r = np.zeros_like(a)
            pg.p3dfft_btran_c2r(c, r, "tff")
            assert orc.normalised_linf(r, ref.btran_c2r(c, "tff")) <= TOL
    finally:
        pg.p3dfft_clean()


@pytest.mark.parametrize("scale", [2.0 ** 800, 2.0 ** -800, 1.0])
def test_dropin_in_place_picks_bias_on_device(torch_cuda, scale):
    # ftran_r2c(B, B) / btran_c2r(B, B) on one device buffer sized by memsize:
    # the input is overwritten, so the call measures it first
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = 16, 16, 16
    mem = pg.p3dfft_setup((1, 1), nx, ny, nz)
    try:
        ref = orc.OraclePlan(nx, ny, nz)
        a = _field((nz, ny, nx), 12, scale)
        buf = torch.zeros(mem[0] * mem[1] * mem[2], dtype=torch.float64, device="cuda")
        buf[: a.size] = torch.from_numpy(a.ravel()).cuda()
        pg.p3dfft_ftran_r2c(buf, buf, "fft")
        want = ref.ftran_r2c(a, "fft")
        got = buf.view(torch.complex128)[: want.size].cpu().numpy().reshape(want.shape)
        assert orc.normalised_linf(got, want) <= TOL
        pg.p3dfft_btran_c2r(buf, buf, "tff")
        back = buf[: a.size].cpu().numpy().reshape(a.shape)
        assert orc.normalised_linf(back, ref.btran_c2r(want, "tff")) <= TOL
    finally:
        pg.p3dfft_clean()


def test_dropin_x_only_and_cheby_at_large_scale(torch_cuda):
    import scipy.fft as sfft

    import p3dfft_gb300 as pg
    nx, ny, nz, lz = 16, 12, 17, 2.0
    a = _field((nz, ny, nx), 13, 1e250)
    pg.p3dfft_setup((1, 1), nx, ny, nz)
    try:
        c1 = np.zeros((nz, ny, nx // 2 + 1), np.complex128)
        pg.p3dfft_ftran_r2c_1d(a, c1)
        assert orc.normalised_linf(c1, sfft.rfft(a, axis=2)) <= TOL
        c = np.zeros((nz, ny, nx // 2 + 1), np.complex128)
        pg.p3dfft_cheby(a, c, lz)
        assert orc.normalised_linf(c, orc.OraclePlan(nx, ny, nz).cheby(a, lz)) <= TOL
    finally:
        pg.p3dfft_clean()


def test_batch_reports_out_of_window_inputs(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    plan = pg.Plan(32, 24, 20, precision=pg.F64)
    x = torch.from_numpy(_field((20, 24, 32), 14, 2.0 ** 700)).cuda()
    out = torch.empty(plan.complex_shape, dtype=torch.complex128, device="cuda")
    b = pg.Batch(pg.F64).set_jobs([{"plan": plan, "kind": pg.JOB_FORWARD, "in": x, "out": out}])
    b.launch()
    with pytest.raises(pg.P3DFFTError, match="exponent window"):
        b.check()
    # in the window, the same batch is clean
    x.mul_(2.0 ** -700)
    b.launch()
    b.check()
    b.close()
    plan.close()
