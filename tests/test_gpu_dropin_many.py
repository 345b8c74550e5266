"""The drop-in library's multi-field and X-only entry points on the GPU,
through libp3dfft.so / libp3dfft_single.so as a reference caller binds them:

* p3dfft_ftran_r2c_many / p3dfft_btran_c2r_many (build/ftran.F90:84-317,
  build/btran.F90:84-304): nv fields spaced dim_in / dim_out elements apart,
  host and device arrays, padded spacings, a pruned grid;
* p3dfft_cheby_many (build/ftran.F90:321-354);
* p3dfft_ftran_r2c_1d (build/ftran.F90:787-814): the X r2c alone.

Tolerances as the other parity tests: F64 normalised L-inf 1e-12, F32
relative L2 1e-6 against the FP64 oracle.
"""
import numpy as np
import pytest
import scipy.fft as sfft

from oracle import p3dfft_oracle as orc

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
F32_TOL = 1e-6


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300  # noqa: F401
    return torch


def _fields(nv, n, pad, seed):
    a = np.zeros((nv, n + pad))
    a[:, :n] = np.random.default_rng(seed).uniform(-1, 1, size=(nv, n))
    return a


@pytest.mark.parametrize("where", ["host", "device"])
@pytest.mark.parametrize("args", [(16, 12, 10), (20, 16, 12, 16, 10, 8), (15, 9, 14)])
def test_dropin_many_fields(torch_cuda, where, args):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = args[:3]
    nxc, nyc, nzc = args[3:] if len(args) > 3 else (nx, ny, nz)
    nv = 3
    rsize = nx * ny * nz
    csize = (nxc // 2 + 1) * nyc * nzc
    dim_in, dim_out = rsize + 7, csize + 5
    a = _fields(nv, rsize, 7, 21)
    ref = orc.OraclePlan(nx, ny, nz, nxc, nyc, nzc)
    want = ref.ftran_many([a[v, :rsize].reshape(nz, ny, nx) for v in range(nv)], "fft")
    pg.p3dfft_setup((1, 1), nx, ny, nz, 0, nxc, nyc, nzc, True)
    try:
        if where == "host":
            x = a.copy()
            b = np.zeros((nv, dim_out), np.complex128)
        else:
            x = torch.from_numpy(a).cuda()
            b = torch.zeros((nv, dim_out), dtype=torch.complex128, device="cuda")
        pg.p3dfft_ftran_r2c_many(x, dim_in, b, dim_out, nv, "fft")
        got = b if where == "host" else b.cpu().numpy()
        for v in range(nv):
            assert orc.normalised_linf(got[v, :csize].reshape(want[v].shape), want[v]) <= F64_TOL
            assert np.all(got[v, csize:] == 0)  # the spacing's padding is not written
        # backward of a seeded spectrum (the padding holds values that must be ignored)
        rng = np.random.default_rng(22)
        c = rng.standard_normal((nv, dim_out)) + 1j * rng.standard_normal((nv, dim_out))
        want_r = ref.btran_many([c[v, :csize].reshape(want[v].shape) for v in range(nv)], "tff")
        if where == "host":
            cin = c.copy()
            r = np.zeros((nv, dim_in))
        else:
            cin = torch.from_numpy(c).cuda()
            r = torch.zeros((nv, dim_in), dtype=torch.float64, device="cuda")
        pg.p3dfft_btran_c2r_many(cin, dim_out, r, dim_in, nv, "tff")
        gr = r if where == "host" else r.cpu().numpy()
        cin_back = cin if where == "host" else cin.cpu().numpy()
        assert np.array_equal(cin_back, c)  # the input is not modified
        for v in range(nv):
            assert orc.normalised_linf(gr[v, :rsize].reshape(nz, ny, nx), want_r[v]) <= F64_TOL
            assert np.all(gr[v, rsize:] == 0)
    finally:
        pg.p3dfft_clean()


def test_dropin_many_single_precision(torch_cuda):
    import p3dfft_gb300 as pg
    nx, ny, nz, nv = 24, 20, 18, 2
    rsize, csize = nx * ny * nz, (nx // 2 + 1) * ny * nz
    a = _fields(nv, rsize, 3, 23).astype(np.float32)
    pg.p3dfft_setup((1, 1), nx, ny, nz, single=True)
    try:
        b = np.zeros((nv, csize + 1), np.complex64)
        pg.p3dfft_ftran_r2c_many(a, rsize + 3, b, csize + 1, nv, "fft")
        ref = orc.OraclePlan(nx, ny, nz)
        for v in range(nv):
            want = ref.ftran_r2c(a[v, :rsize].astype(np.float64).reshape(nz, ny, nx), "fft")
            assert orc.relative_l2(b[v, :csize].reshape(want.shape).astype(np.complex128), want) <= F32_TOL
        b *= 1.0 / rsize
        r = np.zeros_like(a)
        pg.p3dfft_btran_c2r_many(b, csize + 1, r, rsize + 3, nv, "tff")
        for v in range(nv):
            assert np.abs(r[v, :rsize] - a[v, :rsize]).max() <= orc.roundtrip_tolerance(rsize, single=True)
    finally:
        pg.p3dfft_clean()


@pytest.mark.parametrize("where", ["host", "device"])
def test_dropin_cheby_many(torch_cuda, where):
    # driver_cheby.F90's field per variable, with a different amplitude each
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz, nv, lz = 16, 12, 17, 2, 2.0
    rsize, csize = nx * ny * nz, (nx // 2 + 1) * ny * nz
    coord_z = np.cos(np.pi * np.arange(nz) / (nz - 1)) * 2.0 / lz
    a = np.zeros((nv, rsize + 4))
    rng = np.random.default_rng(24)
    for v in range(nv):
        f = np.sin((v + 1) * coord_z)[:, None, None] * (1 + 0.1 * rng.uniform(-1, 1, (nz, ny, nx)))
        a[v, :rsize] = f.ravel()
    ref = orc.OraclePlan(nx, ny, nz)
    pg.p3dfft_setup((1, 1), nx, ny, nz)
    try:
        if where == "host":
            x, b = a.copy(), np.zeros((nv, csize + 2), np.complex128)
        else:
            x = torch.from_numpy(a).cuda()
            b = torch.zeros((nv, csize + 2), dtype=torch.complex128, device="cuda")
        pg.p3dfft_cheby_many(x, rsize + 4, b, csize + 2, nv, lz)
        got = b if where == "host" else b.cpu().numpy()
        for v in range(nv):
            want = ref.cheby(a[v, :rsize].reshape(nz, ny, nx), lz)
            assert orc.normalised_linf(got[v, :csize].reshape(want.shape), want) <= F64_TOL
    finally:
        pg.p3dfft_clean()


@pytest.mark.parametrize("where", ["host", "device"])
@pytest.mark.parametrize("shape", [(32, 16, 8), (15, 9, 7), (64, 6, 5)])
def test_dropin_ftran_r2c_1d(torch_cuda, where, shape):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = shape
    a = np.random.default_rng(25).uniform(-1, 1, (nz, ny, nx))
    want = sfft.rfft(a, axis=2)  # FFTW r2c along x, unnormalised, every mode
    pg.p3dfft_setup((1, 1), nx, ny, nz, 0, nx // 2 * 2 or 1, ny, nz)  # pruning does not apply to the X-only call
    try:
        if where == "host":
            x, c = a.copy(), np.zeros((nz, ny, nx // 2 + 1), np.complex128)
        else:
            x = torch.from_numpy(a).cuda()
            c = torch.zeros((nz, ny, nx // 2 + 1), dtype=torch.complex128, device="cuda")
        pg.p3dfft_ftran_r2c_1d(x, c)
        got = c if where == "host" else c.cpu().numpy()
        assert orc.normalised_linf(got, want) <= F64_TOL
    finally:
        pg.p3dfft_clean()


def test_plan_ftran_r2c_1d_f32(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = 48, 10, 6
    a = np.random.default_rng(26).uniform(-1, 1, (nz, ny, nx)).astype(np.float32)
    plan = pg.Plan(nx, ny, nz, precision=pg.F32)
    c = plan.ftran_r2c_1d(torch.from_numpy(a).cuda()).cpu().numpy()
    want = sfft.rfft(a.astype(np.float64), axis=2)
    assert orc.relative_l2(c.astype(np.complex128), want) <= F32_TOL
    plan.close()
