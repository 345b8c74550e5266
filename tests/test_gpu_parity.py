"""GPU parity of the sm_103a transforms against the CPU oracle (through the C-ABI).

Tolerances: F64 path, normalised L-inf (max|gpu - oracle| / max|oracle|)
<= 1e-12 for forward and backward outputs; F32 path, relative L2 <= 1e-6
against the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import p3dfft_oracle as orc

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
F32_TOL = 1e-6


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300  # noqa: F401  (loads the native libraries; no fallback)
    return torch


def _rand(shape, seed):
    return np.random.default_rng(seed).uniform(-1.0, 1.0, size=shape)


def _spectrum(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


MODES = {"pipe_tma": (True, True), "pipe_cpasync": (True, False), "single_tile": (False, False)}


def _run_pair(torch, plan_args, a, op_f, op_b, precision, seed=0, mode="pipe_tma", stride1=False):
    import p3dfft_gb300 as pg
    nx, ny, nz = plan_args[:3]
    pruned = plan_args[3:] if len(plan_args) > 3 else (nx, ny, nz)
    plan = pg.Plan(nx, ny, nz, *pruned, precision=precision,
                   layout=pg.LAYOUT_STRIDE1 if stride1 else pg.LAYOUT_XYZ)
    plan.set_options(*MODES[mode])
    ref = orc.OraclePlan(nx, ny, nz, *pruned, stride1=stride1)
    rdt = torch.float64 if precision == pg.F64 else torch.float32
    x = torch.from_numpy(a).to("cuda", rdt)
    b = plan.ftran_r2c(x, op=op_f)
    want_b = ref.ftran_r2c(a, op_f)
    c_in = _spectrum(want_b.shape, seed + 1)
    cdt = torch.complex128 if precision == pg.F64 else torch.complex64
    r = plan.btran_c2r(torch.from_numpy(c_in).to("cuda", cdt), op=op_b)
    want_r = ref.btran_c2r(c_in, op_b)
    torch.cuda.synchronize()
    plan.check()
    got_b = b.cpu().numpy().astype(np.complex128)
    got_r = r.cpu().numpy().astype(np.float64)
    plan.close()
    return got_b, want_b, got_r, want_r


SIZES = [
    (32, 32, 32),
    (16, 8, 4),
    (14, 26, 38),    # 7, 13, 19: generic prime stages (the reference's uneven-grid test)
    (15, 9, 7),      # odd lengths everywhere
    (48, 64, 96),
    (120, 160, 192),
    (60, 36, 45),
    (2, 3, 5),
    (1, 4, 6),
    (128, 128, 128),
]


@pytest.mark.parametrize("shape", SIZES)
def test_f64_fft_parity(torch_cuda, shape):
    import p3dfft_gb300 as pg
    a = _rand(shape[::-1], 11)
    gb, wb, gr, wr = _run_pair(torch_cuda, shape, a, "fft", "tff", pg.F64)
    assert orc.normalised_linf(gb, wb) <= F64_TOL
    assert orc.normalised_linf(gr, wr) <= F64_TOL


@pytest.mark.parametrize("shape", [(32, 32, 33), (16, 12, 9), (24, 20, 17), (8, 8, 2)])
@pytest.mark.parametrize("ops", [("ffc", "cff"), ("ffs", "sff"), ("ffn", "nff"), ("fff", "fff")])
def test_f64_z_ops_parity(torch_cuda, shape, ops):
    import p3dfft_gb300 as pg
    a = _rand(shape[::-1], 5)
    gb, wb, gr, wr = _run_pair(torch_cuda, shape, a, ops[0], ops[1], pg.F64)
    assert orc.normalised_linf(gb, wb) <= F64_TOL
    assert orc.normalised_linf(gr, wr) <= F64_TOL


@pytest.mark.parametrize("args", [(64, 64, 64, 32, 32, 32), (16, 12, 10, 8, 6, 4), (16, 16, 16, 10, 9, 7),
                                  (20, 18, 16, 20, 7, 16), (24, 24, 24, 24, 24, 9)])
def test_f64_pruned_parity(torch_cuda, args):
    import p3dfft_gb300 as pg
    a = _rand(args[:3][::-1], 3)
    gb, wb, gr, wr = _run_pair(torch_cuda, args, a, "fft", "tff", pg.F64)
    assert orc.normalised_linf(gb, wb) <= F64_TOL
    assert orc.normalised_linf(gr, wr) <= F64_TOL


@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("case", [((64, 48, 40), "fft", "tff", 0), ((32, 24, 33), "ffc", "cff", 0),
                                  ((16, 12, 10), "ffs", "sff", 0), ((64, 64, 64, 32, 32, 32), "fft", "tff", 0),
                                  ((96, 80, 60), "fft", "tff", 1), ((30, 18, 17), "ffc", "cff", 1),
                                  ((33, 20, 16, 20, 9, 10), "fft", "tff", 1)])
def test_kernel_paths_agree(torch_cuda, mode, case):
    # every kernel family (pipelined TMA, pipelined cp.async, single-tile) on
    # the same cases, F64 (last field 0) and F32 (1)
    import p3dfft_gb300 as pg
    args, op_f, op_b, f32 = case
    a = _rand(args[:3][::-1], 17)
    gb, wb, gr, wr = _run_pair(torch_cuda, args, a, op_f, op_b, pg.F32 if f32 else pg.F64, mode=mode)
    if f32:
        assert orc.relative_l2(gb, wb) <= F32_TOL
        assert orc.relative_l2(gr, wr) <= F32_TOL
    else:
        assert orc.normalised_linf(gb, wb) <= F64_TOL
        assert orc.normalised_linf(gr, wr) <= F64_TOL


@pytest.mark.parametrize("shape", [(32, 32, 32), (14, 26, 38), (120, 160, 192), (128, 128, 128)])
def test_f32_parity(torch_cuda, shape):
    import p3dfft_gb300 as pg
    a = _rand(shape[::-1], 21)
    gb, wb, gr, wr = _run_pair(torch_cuda, shape, a, "fft", "tff", pg.F32)
    assert orc.relative_l2(gb, wb) <= F32_TOL
    assert orc.relative_l2(gr, wr) <= F32_TOL


# binary32 complex rows of nx/2+1 modes start at odd 8-byte elements when
# nx/2+1 is odd: the backward Z pass then reads each plane's positions as its
# columns (TMA) when it can, and phase-shifted tiles otherwise (pruned z, DST,
# unaligned fields, no TMA); every form must match the oracle
@pytest.mark.parametrize("mode", ["pipe_tma", "pipe_cpasync"])
@pytest.mark.parametrize("case", [((64, 48, 40), "fft", "tff"), ((64, 48, 40, 64, 30, 40), "fft", "tff"),
                                  ((64, 48, 40, 64, 48, 30), "fft", "tff"), ((40, 36, 33), "ffc", "cff"),
                                  ((40, 36, 30), "ffs", "sff"), ((96, 20, 64), "fft", "tff")])
def test_f32_odd_row_backward(torch_cuda, mode, case):
    import p3dfft_gb300 as pg
    args, opf, opb = case
    a = _rand(args[:3][::-1], 23)
    gb, wb, gr, wr = _run_pair(torch_cuda, args, a, opf, opb, pg.F32, mode=mode)
    assert orc.relative_l2(gb, wb) <= F32_TOL
    assert orc.relative_l2(gr, wr) <= F32_TOL


@pytest.mark.parametrize("spacing", [0, 1, 2])
def test_f32_odd_row_backward_many_fields(torch_cuda, spacing):
    # field spacings that keep every field 16-byte aligned (0, 2) or not (1)
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz, nv = 64, 24, 40, 3
    plan = pg.Plan(nx, ny, nz, precision=pg.F32)
    ref = orc.OraclePlan(nx, ny, nz)
    csize, rsize = (nx // 2 + 1) * ny * nz, nx * ny * nz
    dim_c, dim_r = csize + spacing, rsize + 2
    c = _spectrum((nv, dim_c), 24)
    r = torch.zeros((nv, dim_r), dtype=torch.float32, device="cuda")
    plan.btran_c2r(torch.from_numpy(c).to("cuda", torch.complex64), r, op="tff", nv=nv, dim_in=dim_c,
                   dim_out=dim_r)
    plan.check()
    got = r.cpu().numpy().astype(np.float64)
    for v in range(nv):
        cv = c[v, :csize].astype(np.complex64).astype(np.complex128).reshape(nz, ny, nx // 2 + 1)
        want = ref.btran_c2r(cv, "tff")
        assert orc.relative_l2(got[v, :rsize].reshape(nz, ny, nx), want) <= F32_TOL
    plan.close()


@pytest.mark.parametrize("chunks", [1, 3, 8])
def test_f32_host_row_blocks_bit_identical(torch_cuda, chunks):
    # row blocks of odd-length binary32 rows start at 16-byte boundaries or
    # not; both load forms give the plain call's bits
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = 64, 21, 18
    plan = pg.Plan(nx, ny, nz, precision=pg.F32)
    c = torch.from_numpy(_spectrum(plan.complex_shape, 25)).to("cuda", torch.complex64)
    want = plan.btran_c2r(c)
    hc = c.cpu().pin_memory()
    r = torch.zeros((nz, ny, nx), dtype=torch.float32, device="cuda")
    plan.btran_c2r_from_host(hc, r, chunks=chunks)
    assert torch.equal(r, want)
    plan.check()
    plan.close()


def test_f64_roundtrip_sample_rule(torch_cuda):
    # driver_rand.F90: ftran 'fft', multiply by 1/N, btran 'tff', max |diff| <= 1e-14 N/4
    import p3dfft_gb300 as pg
    nx = ny = nz = 128
    a = np.random.default_rng(99).random((nz, ny, nx))
    plan = pg.Plan(nx, ny, nz)
    x = torch_cuda.from_numpy(a).cuda()
    b = plan.ftran_r2c(x, op="fft")
    b *= 1.0 / a.size
    r = plan.btran_c2r(b, op="tff")
    err = float((r - x).abs().max())
    assert err <= orc.roundtrip_tolerance(a.size)
    assert err < 1e-13


def test_many_fields(torch_cuda):
    import p3dfft_gb300 as pg
    nx, ny, nz, nv = 16, 12, 10, 3
    plan = pg.Plan(nx, ny, nz)
    ref = orc.OraclePlan(nx, ny, nz)
    rsize = nx * ny * nz
    csize = (nx // 2 + 1) * ny * nz
    dim_in, dim_out = rsize + 5, csize + 3
    a = _rand((nv, dim_in), 8)
    x = torch_cuda.from_numpy(a).cuda()
    out = torch_cuda.zeros((nv, dim_out), dtype=torch_cuda.complex128, device="cuda")
    plan.ftran_r2c(x, out, op="fft", nv=nv, dim_in=dim_in, dim_out=dim_out)
    back = torch_cuda.zeros((nv, dim_in), dtype=torch_cuda.float64, device="cuda")
    plan.btran_c2r(out, back, op="tff", nv=nv, dim_in=dim_out, dim_out=dim_in)
    got = out.cpu().numpy()
    gback = back.cpu().numpy()
    for v in range(nv):
        want = ref.ftran_r2c(a[v, :rsize].reshape(nz, ny, nx), "fft")
        assert orc.normalised_linf(got[v, :csize].reshape(want.shape), want) <= F64_TOL
        assert np.all(got[v, csize:] == 0)  # padding untouched
        wr = ref.btran_c2r(want, "tff")
        assert orc.normalised_linf(gback[v, :rsize].reshape(nz, ny, nx), wr) <= F64_TOL
        assert np.array_equal(gback[v, rsize:], a[v, rsize:] * 0)  # zero-initialised padding untouched


def test_in_place_transform(torch_cuda):
    # ftran_r2c(B, B) / btran_c2r(B, B) on one buffer sized by memsize (driver_sine_inplace)
    import p3dfft_gb300 as pg
    nx, ny, nz = 16, 16, 16
    plan = pg.Plan(nx, ny, nz)
    _, _, mem = plan.get_dims(3)
    buf = torch_cuda.zeros(mem[0] * mem[1] * mem[2], dtype=torch_cuda.float64, device="cuda")
    a = _rand((nz, ny, nx), 4)
    buf[: a.size] = torch_cuda.from_numpy(a.ravel()).cuda()
    plan.ftran_r2c(buf, buf, op="fft")
    want = orc.OraclePlan(nx, ny, nz).ftran_r2c(a, "fft")
    got = buf.view(torch_cuda.complex128)[: want.size].cpu().numpy().reshape(want.shape)
    assert orc.normalised_linf(got, want) <= F64_TOL
    buf.view(torch_cuda.complex128)[: want.size] *= 1.0 / a.size
    plan.btran_c2r(buf, buf, op="tff")
    back = buf[: a.size].cpu().numpy().reshape(a.shape)
    assert np.abs(back - a).max() <= orc.roundtrip_tolerance(a.size)


def test_cheby_known_answer(torch_cuda):
    # driver_cheby.F90 on the device path: d/dz sin(z) on Gauss-Lobatto points
    import p3dfft_gb300 as pg
    nx, ny, nz, lz = 32, 32, 33, 2.0
    coord_z = np.cos(np.pi * np.arange(nz) / (nz - 1)) * 2.0 / lz
    a = np.broadcast_to(np.sin(coord_z)[:, None, None], (nz, ny, nx)).copy()
    plan = pg.Plan(nx, ny, nz)
    c = plan.cheby(torch_cuda.from_numpy(a).cuda(), lz)
    want = orc.OraclePlan(nx, ny, nz).cheby(a, lz)
    assert orc.normalised_linf(c.cpu().numpy(), want) <= F64_TOL
    c[0] *= 2.0
    c[nz - 1] *= 2.0
    c *= 0.5
    r = plan.btran_c2r(c, op="cff").cpu().numpy()
    want_r = orc.OraclePlan(nx, ny, nz).btran_c2r(c.cpu().numpy(), "cff")
    assert orc.normalised_linf(r, want_r) <= F64_TOL
    # the sample's rule (driver_cheby.F90:275-284); the 33-point spectral
    # derivative itself is exact to ~1e-12
    err = np.abs(r - np.cos(coord_z)[:, None, None]).max()
    assert err <= 1e-14 * nx * ny * nz * 0.25 and err < 1e-11


def test_dropin_host_api(torch_cuda):
    # the reference's module interface with host arrays, as driver_rand.c uses it
    import p3dfft_gb300 as pg
    nx, ny, nz = 32, 16, 8
    mem = pg.p3dfft_setup((1, 1), nx, ny, nz, 0, nx, ny, nz, False)
    try:
        assert pg.p3dfft_get_dims(1) == ((1, 1, 1), (nx, ny, nz), (nx, ny, nz))
        s, e, fsize = pg.p3dfft_get_dims(2)
        assert fsize == (nx // 2 + 1, ny, nz)
        assert pg.p3dfft_get_dims(3)[2] == mem
        a = np.random.default_rng(5).random((nz, ny, nx))
        b = np.zeros((nz, ny, nx // 2 + 1), np.complex128)
        pg.p3dfft_ftran_r2c(a, b, "fft")
        want = orc.OraclePlan(nx, ny, nz).ftran_r2c(a, "fft")
        assert orc.normalised_linf(b, want) <= F64_TOL
        b *= 1.0 / a.size
        c = np.zeros_like(a)
        pg.p3dfft_btran_c2r(b, c, "tff")
        assert np.abs(c - a).max() <= orc.roundtrip_tolerance(a.size)
        t = pg.get_timers()
        assert t[4] > 0 and t[6] > 0 and t[7] > 0 and t[8] > 0 and t[9] > 0 and t[11] > 0
        assert t[0] == t[1] == t[2] == t[3] == 0
        with pytest.raises(pg.P3DFFTError):
            pg.p3dfft_ftran_r2c(a, b, "ffq")
    finally:
        pg.p3dfft_clean()
    # timers survive clean (driver_rand.c reads them after Cp3dfft_clean)
    assert pg.get_timers()[4] > 0
    with pytest.raises(pg.P3DFFTError):
        pg.p3dfft_get_dims(1)


def test_dropin_single_precision(torch_cuda):
    import p3dfft_gb300 as pg
    nx, ny, nz = 16, 16, 16
    pg.p3dfft_setup((1, 1), nx, ny, nz, single=True)
    try:
        a = np.random.default_rng(6).random((nz, ny, nx)).astype(np.float32)
        b = np.zeros((nz, ny, nx // 2 + 1), np.complex64)
        pg.p3dfft_ftran_r2c(a, b, "fft")
        want = orc.OraclePlan(nx, ny, nz).ftran_r2c(a.astype(np.float64), "fft")
        assert orc.relative_l2(b, want) <= F32_TOL
        b *= 1.0 / a.size
        c = np.zeros_like(a)
        pg.p3dfft_btran_c2r(b, c, "tff")
        assert np.abs(c - a).max() <= orc.roundtrip_tolerance(a.size, single=True)
    finally:
        pg.p3dfft_clean()


def test_device_pointer_dropin(torch_cuda):
    # device arrays go straight to the kernels (no staging)
    import p3dfft_gb300 as pg
    nx, ny, nz = 16, 12, 10
    pg.p3dfft_setup((1, 1), nx, ny, nz)
    try:
        a = _rand((nz, ny, nx), 12)
        x = torch_cuda.from_numpy(a).cuda()
        b = torch_cuda.zeros((nz, ny, nx // 2 + 1), dtype=torch_cuda.complex128, device="cuda")
        pg.p3dfft_ftran_r2c(x, b, "fft")
        want = orc.OraclePlan(nx, ny, nz).ftran_r2c(a, "fft")
        assert orc.normalised_linf(b.cpu().numpy(), want) <= F64_TOL
    finally:
        pg.p3dfft_clean()


def test_unknown_op_is_an_error(torch_cuda):
    import p3dfft_gb300 as pg
    plan = pg.Plan(8, 8, 8)
    x = torch_cuda.zeros((8, 8, 8), dtype=torch_cuda.float64, device="cuda")
    with pytest.raises(pg.P3DFFTError, match="Unknown transform type"):
        plan.ftran_r2c(x, op="ffx")


# ------------------------------------------------------------ STRIDE1 layout
# (nzc, nyc, nxhpc) in Fortran order, z fastest (module.F90:245-254,
# reorder.F90:359-488): the Z pass stores and loads with z adjacent.

@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("case", [((32, 32, 32), "fft", "tff"), ((14, 26, 38), "fft", "tff"),
                                  ((24, 20, 17), "ffc", "cff"), ((16, 12, 9), "ffs", "sff"),
                                  ((16, 12, 10), "ffn", "nff"), ((64, 64, 64, 32, 32, 32), "fft", "tff"),
                                  ((33, 20, 16, 20, 9, 10), "fft", "tff"), ((96, 80, 60), "fft", "tff")])
def test_stride1_parity(torch_cuda, mode, case):
    import p3dfft_gb300 as pg
    args, op_f, op_b = case
    a = _rand(args[:3][::-1], 23)
    gb, wb, gr, wr = _run_pair(torch_cuda, args, a, op_f, op_b, pg.F64, mode=mode, stride1=True)
    assert gb.shape == wb.shape
    assert orc.normalised_linf(gb, wb) <= F64_TOL
    assert orc.normalised_linf(gr, wr) <= F64_TOL


@pytest.mark.parametrize("args", [(48, 64, 96), (30, 18, 17, 30, 9, 10)])
def test_stride1_f32(torch_cuda, args):
    import p3dfft_gb300 as pg
    a = _rand(args[:3][::-1], 29)
    gb, wb, gr, wr = _run_pair(torch_cuda, args, a, "fft", "tff", pg.F32, stride1=True)
    assert orc.relative_l2(gb, wb) <= F32_TOL
    assert orc.relative_l2(gr, wr) <= F32_TOL


def test_stride1_cheby_and_dims(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = 16, 12, 17
    plan = pg.Plan(nx, ny, nz, precision=pg.F64, layout=pg.LAYOUT_STRIDE1)
    ref = orc.OraclePlan(nx, ny, nz, stride1=True)
    assert plan.get_dims(2) == ref.get_dims(2)
    z = np.cos(np.pi * np.arange(nz) / (nz - 1))
    a = np.cos(2 * np.pi * np.arange(nx) / nx)[None, None, :] * z[:, None, None] ** 3 * np.ones((1, ny, 1))
    got = plan.cheby(torch.from_numpy(a).cuda(), 2.0).cpu().numpy()
    want = ref.cheby(a, 2.0)
    plan.close()
    assert got.shape == want.shape == (nx // 2 + 1, ny, nz)
    assert orc.normalised_linf(got, want) <= F64_TOL


def test_stride1_drop_in(torch_cuda):
    import p3dfft_gb300 as pg
    nx, ny, nz = 24, 16, 10
    a = _rand((nz, ny, nx), 31)
    pg.p3dfft_setup((1, 1), nx, ny, nz, stride1=True)
    try:
        s, e, sz = pg.p3dfft_get_dims(2)
        assert sz == (nz, ny, nx // 2 + 1)
        b = np.zeros((nx // 2 + 1, ny, nz), dtype=np.complex128)
        pg.p3dfft_ftran_r2c(a, b, "fft")
        r = np.zeros_like(a)
        pg.p3dfft_btran_c2r(b, r, "tff")
    finally:
        pg.p3dfft_clean()
    ref = orc.OraclePlan(nx, ny, nz, stride1=True)
    assert orc.normalised_linf(b, ref.ftran_r2c(a, "fft")) <= F64_TOL
    assert np.max(np.abs(r / (nx * ny * nz) - a)) <= orc.roundtrip_tolerance(nx * ny * nz)


_HOST_PATH_SCRIPT = r"""
import sys, numpy as np, torch
import p3dfft_gb300 as pg
nx, ny, nz = 48, 40, 36
a = np.random.default_rng(3).uniform(-1, 1, (nz, ny, nx))
out = {}
pg.p3dfft_setup((1, 1), nx, ny, nz)
b = np.zeros((nz, ny, nx // 2 + 1), dtype=np.complex128)       # pageable host arrays
pg.p3dfft_ftran_r2c(a, b, "fft")
r = np.zeros_like(a)
pg.p3dfft_btran_c2r(b, r, "tff")
pa = torch.from_numpy(a).pin_memory()                              # page-locked host arrays
pb = torch.zeros((nz, ny, nx // 2 + 1), dtype=torch.complex128).pin_memory()
pr = torch.zeros((nz, ny, nx), dtype=torch.float64).pin_memory()
pg.p3dfft_ftran_r2c(pa, pb, "ffc")
pg.p3dfft_btran_c2r(pb, pr, "cff")
pg.p3dfft_clean()
np.savez(sys.argv[1], b=b, r=r, pb=pb.numpy(), pr=pr.numpy())
"""


@pytest.mark.parametrize("direct", ["1", "0"])
def test_host_arrays_direct_and_staged(torch_cuda, tmp_path, direct):
    # host arrays reached by the kernels in place (P3DFFT_GB_HOST_DIRECT=1,
    # the default where the GPU can address them) or staged through device
    # buffers (=0): the same results, matching the oracle
    import os
    import subprocess
    import sys
    f = tmp_path / "out.npz"
    env = dict(os.environ, P3DFFT_GB_HOST_DIRECT=direct)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.run([sys.executable, "-c", _HOST_PATH_SCRIPT, str(f)], check=True, env=env, cwd=root, timeout=300)
    d = np.load(f)
    nx, ny, nz = 48, 40, 36
    a = np.random.default_rng(3).uniform(-1, 1, (nz, ny, nx))
    ref = orc.OraclePlan(nx, ny, nz)
    assert orc.normalised_linf(d["b"], ref.ftran_r2c(a, "fft")) <= F64_TOL
    assert orc.normalised_linf(d["r"], ref.btran_c2r(ref.ftran_r2c(a, "fft"), "tff")) <= F64_TOL
    assert orc.normalised_linf(d["pb"], ref.ftran_r2c(a, "ffc")) <= F64_TOL
    assert orc.normalised_linf(d["pr"], ref.btran_c2r(ref.ftran_r2c(a, "ffc"), "cff")) <= F64_TOL


@pytest.mark.parametrize("real_on_host", [False, True])
@pytest.mark.parametrize("chunks", [1, 3, 8, 100])
@pytest.mark.parametrize("args", [(48, 40, 36), (33, 20, 16, 20, 9, 10), (16, 12, 3)])
def test_host_row_block_transforms(torch_cuda, args, chunks, real_on_host):
    # p3g_ftran_r2c_to_host / p3g_btran_c2r_from_host: the Z pass in row
    # blocks with the host copies overlapped (and, with the real array in host
    # memory, the X and Y passes in z-slabs on two streams); bit-identical to
    # the plain calls
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = args[:3]
    plan = pg.Plan(*args, precision=pg.F64)
    x = torch.from_numpy(_rand((nz, ny, nx), 41)).cuda()
    want_b = plan.ftran_r2c(x)
    want_r = plan.btran_c2r(want_b)
    xin = x.cpu().pin_memory() if real_on_host else x
    hb = torch.zeros(plan.complex_shape, dtype=torch.complex128).pin_memory()
    plan.ftran_r2c_to_host(xin, hb, chunks=chunks)
    assert torch.equal(hb, want_b.cpu())
    r = torch.zeros((nz, ny, nx), dtype=torch.float64).pin_memory() if real_on_host else torch.zeros_like(x)
    plan.btran_c2r_from_host(hb, r, chunks=chunks)
    assert torch.equal(r.cpu(), want_r.cpu())
    plan.check()
    plan.close()


@pytest.mark.parametrize("case", [((4096, 6, 4), "f64"), ((6, 4096, 4), "f64"), ((4, 6, 4096), "f64"),
                                  ((8192, 4, 2), "f32"), ((4, 2, 8192), "f32")])
def test_longest_lines(torch_cuda, case):
    # the longest lines one tile holds: 4096 points on the F64 path, 8192 on F32
    import p3dfft_gb300 as pg
    shape, prec = case
    a = _rand(shape[::-1], 43)
    if prec == "f64":
        gb, wb, gr, wr = _run_pair(torch_cuda, shape, a, "fft", "tff", pg.F64)
        assert orc.normalised_linf(gb, wb) <= F64_TOL
        assert orc.normalised_linf(gr, wr) <= F64_TOL
    else:
        gb, wb, gr, wr = _run_pair(torch_cuda, shape, a, "fft", "tff", pg.F32)
        assert orc.relative_l2(gb, wb) <= F32_TOL
        assert orc.relative_l2(gr, wr) <= F32_TOL


# Y and Z lines longer than one tile (4096 points F64, 8192 F32) run as
# four-step passes (two launches through a scratch field, n = n1 n2)
@pytest.mark.parametrize("case", [((6, 16384, 4), "f64", False), ((4, 6, 12288), "f64", False),
                                  ((8, 8192, 6), "f64", True), ((10, 6, 10000), "f64", False),
                                  ((4, 16384, 4), "f32", False), ((6, 4, 24576), "f32", True),
                                  ((8192, 6, 4), "f64", False), ((8192, 5, 3), "f64", True),
                                  ((12000, 4, 6), "f64", False), ((16384, 6, 4), "f32", False),
                                  ((10240, 3, 3), "f32", False)])
def test_long_lines_four_step(torch_cuda, case):
    import p3dfft_gb300 as pg
    shape, prec, stride1 = case
    a = _rand(shape[::-1], 44)
    p = pg.F64 if prec == "f64" else pg.F32
    gb, wb, gr, wr = _run_pair(torch_cuda, shape, a, "fft", "tff", p, stride1=stride1)
    if prec == "f64":
        assert orc.normalised_linf(gb, wb) <= F64_TOL
        assert orc.normalised_linf(gr, wr) <= F64_TOL
    else:
        assert orc.relative_l2(gb, wb) <= F32_TOL
        assert orc.relative_l2(gr, wr) <= F32_TOL


def test_long_lines_many_fields(torch_cuda):
    # nv fields: the four-step passes run field after field
    import p3dfft_gb300 as pg
    nx, ny, nz, nv = 4, 5000, 6, 3
    plan = pg.Plan(nx, ny, nz)
    ref = orc.OraclePlan(nx, ny, nz)
    a = _rand((nv, nz, ny, nx), 45)
    b = plan.ftran_r2c(torch_cuda.from_numpy(a).cuda(), nv=nv).cpu().numpy()
    for v in range(nv):
        assert orc.normalised_linf(b[v], ref.ftran_r2c(a[v], "fft")) <= F64_TOL
    plan.close()


@pytest.mark.parametrize("args", [(4, 8192, 4, 4, 6000, 4), (4, 4, 16384, 4, 4, 9000)])
def test_too_long_lines_are_rejected(torch_cuda, args):
    # pruned y or z lines beyond one tile are refused
    import p3dfft_gb300 as pg
    with pytest.raises(pg.P3DFFTError, match="too long|unsupported"):
        pg.Plan(*args, precision=pg.F64)


def test_tile_wait_times_out_and_context_survives(torch_cuda):
    # the TMA tile barriers of the pipelined passes expect more bytes than
    # their copies deliver (a host-side test hook; nothing faults): every wait
    # runs out, the pass ends early, the status reports the time-out once, and
    # the next transform on the same plan and context is correct
    import time

    import p3dfft_gb300 as pg
    nx, ny, nz = 64, 48, 40
    plan = pg.Plan(nx, ny, nz)
    a = _rand((nz, ny, nx), 46)
    x = torch_cuda.from_numpy(a).cuda()
    plan.block_tiles(True)
    t = time.perf_counter()
    plan.ftran_r2c(x)
    with pytest.raises(pg.P3DFFTError, match="timed out"):
        plan.check()
    assert time.perf_counter() - t < 60
    plan.block_tiles(False)
    b = plan.ftran_r2c(x)
    plan.check()
    assert orc.normalised_linf(b.cpu().numpy(), orc.OraclePlan(nx, ny, nz).ftran_r2c(a, "fft")) <= F64_TOL
    plan.close()
