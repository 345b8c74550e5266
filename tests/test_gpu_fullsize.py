"""Full-size checks through size-independent properties (the configured
workloads are too large for the CPU oracle to finish in seconds):

* 1024^3 and 768x1024x540 FP64: round trip within the samples' pass rule
  (driver_rand.F90:264-276: max error <= 1e-14 N / 4 after the 1/N scaling)
  and Parseval for the forward spectrum;
* linearity of the forward transform (T(a x + b y) = a T x + b T y);
* FP32 against FP64 on the same field (relative L2 <= 1e-6);
* 512x512x257 with the Chebyshev (DCT-I) Z transform: 'ffc' / 'cff' round trip
  scaled by 1/(nx ny 2 (nz - 1)).
"""
import math

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300  # noqa: F401
    return torch


def _field(torch, shape, seed, dtype):
    nx, ny, nz = shape
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return torch.rand((nz, ny, nx), generator=g, device="cuda", dtype=torch.float64).mul_(2).sub_(1).to(dtype)


def _parseval(torch, x, b, nx):
    # sum |x|^2 = (1/N) sum over the full spectrum; the r2c half counts modes
    # 0 < kx < nx/2 twice
    n = x.numel()
    w = torch.ones(b.shape[-1], dtype=torch.float64, device=b.device) * 2.0
    w[0] = 1.0
    if nx % 2 == 0:
        w[-1] = 1.0
    e_spec = float(((b.real.double() ** 2 + b.imag.double() ** 2) * w).sum()) / n
    e_x = float((x.double() ** 2).sum())
    return abs(e_spec - e_x) / e_x


@pytest.mark.parametrize("shape", [(1024, 1024, 1024), (768, 1024, 540)])
def test_fullsize_roundtrip_parseval_linearity(torch_cuda, shape):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = shape
    n = nx * ny * nz
    plan = pg.Plan(nx, ny, nz, precision=pg.F64)
    x = _field(torch, shape, 1, torch.float64)
    b = plan.ftran_r2c(x)
    assert _parseval(torch, x, b, nx) <= 1e-12
    r = plan.btran_c2r(b)
    r.mul_(1.0 / n)
    err = float((r - x).abs().max())
    assert err <= 1e-14 * n * 0.25  # the samples' rule
    assert err <= 1e-12
    del r
    # linearity: T(2x + 3y) = 2 T x + 3 T y
    y = _field(torch, shape, 2, torch.float64)
    by = plan.ftran_r2c(y)
    bxy = plan.ftran_r2c(x.mul_(2.0).add_(y, alpha=3.0))
    d = bxy.sub_(b.mul_(2.0)).sub_(by.mul_(3.0))
    assert float(d.abs().max()) <= 1e-12 * float(by.abs().max()) * 5
    plan.check()
    plan.close()


def test_fullsize_f32_against_f64(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda
    shape = (768, 1024, 540)
    p64 = pg.Plan(*shape, precision=pg.F64)
    p32 = pg.Plan(*shape, precision=pg.F32)
    x = _field(torch, shape, 3, torch.float64)
    b64 = p64.ftran_r2c(x)
    b32 = p32.ftran_r2c(x.float())
    rel = float(torch.linalg.vector_norm(b32.to(torch.complex128) - b64) / torch.linalg.vector_norm(b64))
    assert rel <= 1e-6
    p64.close()
    p32.close()


def test_chebyshev_config_roundtrip(torch_cuda):
    # 512 x 512 x 257, z on the Gauss-Lobatto points, f = sum of 16 seeded
    # sin(2 pi a x) cos(2 pi b y) T_m(z), a, b <= 64, m <= 128, plus noise
    import numpy as np

    import p3dfft_gb300 as pg
    torch = torch_cuda
    nx, ny, nz = 512, 512, 257
    rng = np.random.default_rng(8)
    xs = torch.arange(nx, device="cuda", dtype=torch.float64) / nx
    ys = torch.arange(ny, device="cuda", dtype=torch.float64) / ny
    zs = torch.cos(math.pi * torch.arange(nz, device="cuda", dtype=torch.float64) / (nz - 1))
    f = torch.zeros((nz, ny, nx), dtype=torch.float64, device="cuda")
    for _ in range(16):
        a, b, m = int(rng.integers(0, 65)), int(rng.integers(0, 65)), int(rng.integers(0, 129))
        tz = torch.cos(m * torch.arccos(zs.clamp(-1, 1)))  # T_m on the Lobatto points
        f += (torch.sin(2 * math.pi * a * xs)[None, None, :] * torch.cos(2 * math.pi * b * ys)[None, :, None]
              * tz[:, None, None])
    g = torch.Generator(device="cuda")
    g.manual_seed(9)
    f += 1e-6 * (torch.rand(f.shape, generator=g, device="cuda", dtype=torch.float64) * 2 - 1)
    plan = pg.Plan(nx, ny, nz, precision=pg.F64)
    c = plan.ftran_r2c(f, op="ffc")
    r = plan.btran_c2r(c, op="cff")
    r.mul_(1.0 / (nx * ny * 2 * (nz - 1)))
    err = float((r - f).abs().max()) / float(f.abs().max())
    assert err <= 1e-12
    plan.close()
