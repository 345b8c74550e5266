"""Pins the CPU oracle against the reference's own checks (no GPU).

The reference ships no golden data; its sample programs check results against
analytic answers.  Each test below restates one of those checks and applies it
to the oracle, with the sample's own pass rule where it has one.
"""
import numpy as np
import pytest
import scipy.fft as sfft

from oracle import p3dfft_oracle as orc


def test_fftw_conventions_match_pocketfft():
    """FFTW REDFT00/RODFT00 definitions and c2r DC/Nyquist handling."""
    rng = np.random.default_rng(1)
    n = 9
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    redft00 = np.array([x[0] + (-1) ** k * x[n - 1]
                        + 2 * sum(x[j] * np.cos(np.pi * j * k / (n - 1)) for j in range(1, n - 1))
                        for k in range(n)])
    assert np.abs(sfft.dct(x, type=1) - redft00).max() < 1e-13
    rodft00 = np.array([2 * sum(x[j] * np.sin(np.pi * (j + 1) * (k + 1) / (n + 1)) for j in range(n))
                        for k in range(n)])
    assert np.abs(sfft.dst(x, type=1) - rodft00).max() < 1e-13
    c = rng.standard_normal(5) + 1j * rng.standard_normal(5)
    c0 = c.copy()
    c0[0] = c0[0].real
    c0[-1] = c0[-1].real
    assert np.array_equal(sfft.irfft(c, 8), sfft.irfft(c0, 8))


def test_map_data_to_proc_blocks():
    # setup.F90:608-635: sizes differ by at most one, larger blocks last, full cover
    for data in (1, 7, 14, 26, 38, 65, 128, 513):
        for proc in (1, 2, 3, 4, 5):
            if proc > data:
                continue
            st, en, sz = orc.map_data_to_proc(data, proc)
            assert st[0] == 1 and en[-1] == data
            assert all(en[i] - st[i] + 1 == sz[i] for i in range(proc))
            assert all(st[i + 1] == en[i] + 1 for i in range(proc - 1))
            assert max(sz) - min(sz) <= 1 and sz == sorted(sz)
    assert orc.map_data_to_proc(10, 4) == ([1, 3, 5, 8], [2, 4, 7, 10], [2, 2, 3, 3])


def test_get_dims_1x1_and_2x2_tile_the_grid():
    nx, ny, nz = 14, 26, 38
    p = orc.OraclePlan(nx, ny, nz)
    assert p.get_dims(1) == ((1, 1, 1), (nx, ny, nz), (nx, ny, nz))
    assert p.get_dims(2) == ((1, 1, 1), (nx // 2 + 1, ny, nz), (nx // 2 + 1, ny, nz))
    s1 = orc.OraclePlan(nx, ny, nz, stride1=True)
    assert s1.get_dims(2) == ((1, 1, 1), (nz, ny, nx // 2 + 1), (nz, ny, nx // 2 + 1))
    # 2x2: the four ranks' ip=1 and ip=2 blocks tile the global arrays exactly once
    real_cover = np.zeros((nz, ny, nx), int)
    cplx_cover = np.zeros((nz, ny, nx // 2 + 1), int)
    for rank in range(4):
        q = orc.OraclePlan(nx, ny, nz, dims=(2, 2), rank=rank)
        s, e, z = q.get_dims(1)
        real_cover[s[2] - 1:e[2], s[1] - 1:e[1], s[0] - 1:e[0]] += 1
        assert z == tuple(e[i] - s[i] + 1 for i in range(3))
        s, e, z = q.get_dims(2)
        cplx_cover[s[2] - 1:e[2], s[1] - 1:e[1], s[0] - 1:e[0]] += 1
    assert (real_cover == 1).all() and (cplx_cover == 1).all()


def test_memsize_padding():
    # setup.F90:579-603 at 1x1: memsize = (nx, ny, nz + padi)
    p = orc.OraclePlan(32, 32, 32)
    pad1 = 2 * 32 * 32 * 17 - 32 * 32 * 32
    padi = -(-pad1 // (32 * 32))
    assert p.memsize == (32, 32, 32 + padi)
    assert p.get_dims(3) == ((0, 0, 0), p.memsize, p.memsize)


def _sine_field(nx, ny, nz):
    # driver_sine.F90:322-355
    twopi = 8 * np.arctan(1.0)
    sx = np.sin(np.arange(nx) * twopi / nx)
    sy = np.sin(np.arange(ny) * twopi / ny)
    sz = np.sin(np.arange(nz) * twopi / nz)
    return sz[:, None, None] * sy[None, :, None] * sx[None, None, :]


@pytest.mark.parametrize("shape", [(32, 32, 32), (128, 128, 128), (14, 26, 38)])
def test_sine_known_answer(shape):
    nx, ny, nz = shape
    p = orc.OraclePlan(nx, ny, nz)
    a = _sine_field(nx, ny, nz)
    b = p.ftran_r2c(a, "fft")
    # analytic spectrum: each sin(2 pi j/n) has -i n/2 at k=1 and +i n/2 at k=n-1
    def ax(n, k):
        return np.where(k == 1, -0.5j * n, np.where(k == n - 1, 0.5j * n, 0))
    kz = np.arange(nz)[:, None, None]
    ky = np.arange(ny)[None, :, None]
    kx = np.arange(nx // 2 + 1)[None, None, :]
    expect = ax(nz, kz) * ax(ny, ky) * ax(nx, kx)
    n = nx * ny * nz
    assert np.abs(b - expect).max() <= 1e-12 * n
    # the sample's round-trip rule (driver_sine.F90:282-319)
    c = p.btran_c2r(b / n, "tff")
    assert np.abs(c - a).max() <= orc.roundtrip_tolerance(n)


def test_inverse_four_spikes():
    # driver_inverse.F90: complex wave (init_wave2) -> btran 'tff' -> +-N/4 at four points
    nx, ny, nz = 32, 32, 32
    p = orc.OraclePlan(nx, ny, nz, overwrite=False)
    twopi = 8 * np.arctan(1.0)
    x = np.arange(nx // 2 + 1)
    y = np.arange(ny)
    z = np.arange(nz)
    wave = ((np.cos(x * twopi / nx) + 1j * np.sin(x * twopi / nx))[None, None, :]
            * np.sin(y * 2.0 * twopi / ny)[None, :, None]
            * np.sin(z * 3.0 * twopi / nz)[:, None, None])
    fin = p.btran_c2r(wave, "tff")
    n = nx * ny * nz
    expect = np.zeros_like(fin)
    # Fortran (Nx,3,4) -(N/4), (Nx,3,Nz-2) +, (Nx,Ny-1,4) +, (Nx,Ny-1,Nz-2) -
    expect[3, 2, nx - 1] = -n * 0.25
    expect[nz - 3, 2, nx - 1] = n * 0.25
    expect[3, ny - 2, nx - 1] = n * 0.25
    expect[nz - 3, ny - 2, nx - 1] = -n * 0.25
    assert np.abs(fin - expect).max() <= orc.roundtrip_tolerance(n)


def test_cheby_derivative():
    # driver_cheby.F90:96-111,218-284: d/dz sin(z) on Gauss-Lobatto points
    nx, ny, nz = 32, 32, 33
    lz = 2.0
    p = orc.OraclePlan(nx, ny, nz, overwrite=False)
    coord_z = np.cos(np.pi * np.arange(nz) / (nz - 1)) * 2.0 / lz
    a = np.broadcast_to(np.sin(coord_z)[:, None, None], (nz, ny, nx)).copy()
    c = p.cheby(a, lz)
    c[0] *= 2.0
    c[nz - 1] *= 2.0
    c *= 0.5
    r = p.btran_c2r(c, "cff")
    err = np.abs(r - np.cos(coord_z)[:, None, None]).max()
    assert err <= 1e-14 * nx * ny * nz * 0.25
    assert err < 1e-12


def test_noop_z():
    # driver_noop.F90: 'ffn' forward, 1/(nx*ny), 'nff' backward
    nx, ny, nz = 16, 12, 10
    p = orc.OraclePlan(nx, ny, nz)
    a = _sine_field(nx, ny, nz) + 0.25
    b = p.ftran_r2c(a, "ffn")
    np.testing.assert_allclose(b, sfft.fft(sfft.rfft(a, axis=2), axis=1), atol=1e-12)
    c = p.btran_c2r(b / (nx * ny), "nff")
    assert np.abs(c - a).max() <= orc.roundtrip_tolerance(nx * ny * nz)


@pytest.mark.parametrize("shape", [(32, 32, 32), (14, 26, 38), (15, 9, 7)])
def test_random_roundtrip(shape):
    # driver_rand.F90:180-276 with a seeded generator
    nx, ny, nz = shape
    rng = np.random.default_rng(1234)
    a = rng.random((nz, ny, nx))
    p = orc.OraclePlan(nx, ny, nz)
    b = p.ftran_r2c(a, "fft")
    np.testing.assert_allclose(b, np.fft.rfftn(a), atol=1e-10)
    c = p.btran_c2r(b / a.size, "tff")
    assert np.abs(c - a).max() <= orc.roundtrip_tolerance(a.size)


def test_pruned_matches_mode_selection():
    # driver_sine_pruned: 64^3 grid keeping 32^3 modes; the kept modes are the
    # low nxhpc x-modes, the low nycph/nzcph and top nyc-nycph/nzc-nzcph y/z modes
    nx = ny = nz = 64
    nxc = nyc = nzc = 32
    rng = np.random.default_rng(7)
    a = rng.random((nz, ny, nx))
    full = np.fft.rfftn(a)
    p = orc.OraclePlan(nx, ny, nz, nxc, nyc, nzc)
    b = p.ftran_r2c(a, "fft")
    assert b.shape == (nzc, nyc, nxc // 2 + 1)
    yk = np.r_[0:16, ny - 16:ny]
    zk = np.r_[0:16, nz - 16:nz]
    np.testing.assert_allclose(b, full[np.ix_(zk, yk, np.arange(17))], atol=1e-10)
    # backward zero-fills the dropped modes
    fill = np.zeros_like(full)
    fill[np.ix_(zk, yk, np.arange(17))] = b
    np.testing.assert_allclose(p.btran_c2r(b, "tff"), np.fft.irfftn(fill, s=(nz, ny, nx), axes=(0, 1, 2)) * a.size,
                               atol=1e-9)


def test_dct_and_dst_z_roundtrip():
    nx, ny, nz = 8, 6, 9
    rng = np.random.default_rng(3)
    a = rng.random((nz, ny, nx))
    p = orc.OraclePlan(nx, ny, nz)
    for op_f, op_b, scale in (("ffc", "cff", 2 * (nz - 1)), ("ffs", "sff", 2 * (nz + 1))):
        b = p.ftran_r2c(a, op_f)
        c = p.btran_c2r(b, op_b) / (nx * ny * scale)
        assert np.abs(c - a).max() < 1e-13


def test_spectrum_of_sine_field():
    nx = ny = nz = 32
    p = orc.OraclePlan(nx, ny, nz)
    b = p.ftran_r2c(_sine_field(nx, ny, nz), "fft") / (nx * ny * nz)
    e = orc.shell_spectrum(b, nx, ny, nz)
    assert e.shape[0] == int(np.sqrt(3 * 32 * 32) * 0.5 + 0.5) + 1
    # k = (1, +-1, +-1): k^2 = 3, shell int(sqrt(3)+0.5) = 2, four stored entries of |B| = 1/8
    expect = np.zeros_like(e)
    expect[2] = 3 * 4 / 64.0
    np.testing.assert_allclose(e, expect, atol=1e-14)


@pytest.mark.parametrize("shape", [(16, 12, 10), (15, 9, 7)])
def test_power_spectrum_parseval(shape):
    # unit weights with the conjugate half counted: sum_k E(k) = sum |x|^2 / N
    nx, ny, nz = shape
    a = np.random.default_rng(2).uniform(-1, 1, size=(nz, ny, nx))
    p = orc.OraclePlan(nx, ny, nz)
    b = p.ftran_r2c(a, "fft") / (nx * ny * nz)
    e = orc.shell_spectrum(b, nx, ny, nz, k2_weight=False, hermitian=True)
    assert abs(e.sum() - np.sum(a * a) / (nx * ny * nz)) <= 1e-14
    # a kmax below the largest shell drops the outer modes
    e5 = orc.shell_spectrum(b, nx, ny, nz, k2_weight=False, hermitian=True, kmax=5)
    np.testing.assert_allclose(e5, e[:6], rtol=0, atol=0)


def test_invalid_inputs_raise():
    with pytest.raises(orc.OracleError):
        orc.OraclePlan(0, 4, 4)
    p = orc.OraclePlan(4, 4, 4)
    with pytest.raises(orc.OracleError):
        p.ftran_r2c(np.zeros((4, 4, 4)), "ffx")
    with pytest.raises(orc.OracleError):
        p.btran_c2r(np.zeros((4, 4, 3), complex), "qff")
