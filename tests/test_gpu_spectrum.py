"""GPU shell spectrum (p3g_spectrum) against the oracle's restatement of the
spectrum sample's compute_spectrum (driver_spec.F90:263-341).

Tolerance: normalised L-inf <= 1e-12 over the bins (binary64 accumulation
in a different order than the sample's sequential loop).
"""
import numpy as np
import pytest

from oracle import p3dfft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300  # noqa: F401
    return torch


def _forward(torch, args, precision, stride1, seed, nv=1):
    import p3dfft_gb300 as pg
    nx, ny, nz = args[:3]
    pruned = args[3:] if len(args) > 3 else (nx, ny, nz)
    plan = pg.Plan(nx, ny, nz, *pruned, precision=precision,
                   layout=pg.LAYOUT_STRIDE1 if stride1 else pg.LAYOUT_XYZ)
    rdt = torch.float64 if precision == pg.F64 else torch.float32
    a = np.random.default_rng(seed).uniform(-1, 1, size=((nv,) if nv > 1 else ()) + (nz, ny, nx))
    x = torch.from_numpy(a).to("cuda", rdt)
    b = plan.ftran_r2c(x, op="fft", nv=nv)
    return plan, b


@pytest.mark.parametrize("stride1", [False, True])
@pytest.mark.parametrize("args", [(32, 32, 32), (24, 20, 18), (15, 9, 7), (64, 48, 40, 40, 30, 24), (128, 96, 64)])
def test_spectrum_sample_weighting(torch_cuda, args, stride1):
    import p3dfft_gb300 as pg
    nx, ny, nz = args[:3]
    plan, b = _forward(torch_cuda, args, pg.F64, stride1, 3)
    scale = 1.0 / (nx * ny * nz)
    e = plan.spectrum(b, scale=scale).cpu().numpy()
    plan.check()
    plan.close()
    want = orc.shell_spectrum(b.cpu().numpy() * scale, nx, ny, nz, stride1=stride1)
    assert e.shape == want.shape
    assert orc.normalised_linf(e, want) <= TOL


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("args", [(48, 40, 36), (33, 20, 17)])
def test_power_spectrum_hermitian(torch_cuda, args, precision):
    import p3dfft_gb300 as pg
    nx, ny, nz = args
    prec = pg.F64 if precision == "f64" else pg.F32
    plan, b = _forward(torch_cuda, args, prec, False, 5)
    e = plan.spectrum(b, flags=pg.SPEC_HERMITIAN).cpu().numpy()
    plan.close()
    bh = b.cpu().numpy().astype(np.complex128)
    want = orc.shell_spectrum(bh, nx, ny, nz, k2_weight=False, hermitian=True)
    assert orc.normalised_linf(e, want) <= TOL


def test_spectrum_many_fields_and_kmax(torch_cuda):
    import p3dfft_gb300 as pg
    nx, ny, nz = 40, 36, 30
    plan, b = _forward(torch_cuda, (nx, ny, nz), pg.F64, False, 7, nv=3)
    # kmax = 26 passes the sample's check (4 kmax^2 >= 20^2 + 35^2 + 29^2) but
    # the outermost modes (|k| up to 30.8) fall beyond it and are dropped
    e = plan.spectrum(b, nv=3, kmax=26).cpu().numpy()
    bh = b.cpu().numpy()
    for f in range(3):
        want = orc.shell_spectrum(bh[f], nx, ny, nz, kmax=26)
        assert orc.normalised_linf(e[f], want) <= TOL
    with pytest.raises(pg.P3DFFTError, match="kmax"):
        plan.spectrum(b, nv=3, kmax=5)
    plan.close()


def test_spectrum_single_mode_known_answer(torch_cuda):
    # one Fourier mode cos(2 pi (3x/nx + 2y/ny)): all weight in shell
    # int(sqrt(13) + 0.5) = 4, E = 13 * 2 * (1/2)^2 with the 1/N scaling
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = 32, 16, 8
    x = np.arange(nx)[None, None, :] / nx
    y = np.arange(ny)[None, :, None] / ny
    a = np.cos(2 * np.pi * (3 * x + 2 * y)) * np.ones((nz, 1, 1))
    plan = pg.Plan(nx, ny, nz, precision=pg.F64)
    b = plan.ftran_r2c(torch.from_numpy(a).cuda())
    e = plan.spectrum(b, scale=1.0 / (nx * ny * nz), flags=pg.SPEC_K2 | pg.SPEC_HERMITIAN).cpu().numpy()
    plan.close()
    want = np.zeros_like(e)
    want[4] = 13 * 2 * 0.25
    assert np.max(np.abs(e - want)) <= 1e-13
