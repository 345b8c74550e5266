"""Full-size checks of the configured workloads.

Against the CPU oracle on every host core (numpy/scipy FP64, a few seconds
per direction at these sizes), with the workloads' own seeded fields:

* 768x1024x540, 32 Fourier modes + N(0,1e-3) noise: F64 forward and backward
  (normalised L-inf <= 1e-12), F32 forward and backward (relative L2 <= 1e-6),
  the round trip under the samples' rule (driver_rand.F90:264-276) and every
  seeded mode against its analytic amplitude;
* 512x512x257 with the Chebyshev (DCT-I) Z transform: 'ffc' / 'cff' and
  p3dfft_cheby (ftran.F90:383-464).

Through size-independent properties at 1024^3 and 768x1024x540: Parseval,
the round trip, linearity (T(a x + b y) = a T x + b T y), and FP32 against
FP64 on the same field.
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


def _bench():
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench
    return bench


def _against_oracle(torch, name, seed):
    import p3dfft_gb300 as pg
    bench = _bench()
    cfg = bench.CONFIGS[name]
    grid, ops = cfg["grid"], cfg["ops"]
    p64 = pg.Plan(*grid, precision=pg.F64)
    p32 = pg.Plan(*grid, precision=pg.F32)
    x = bench.make_input(torch, grid, seed, torch.device("cuda"), cfg["input"])
    err = bench.accuracy(torch, grid, ops, cfg["input"], x, p64, p32, None,
                         lz=2.0 if name == "cheby" else None, seed=seed)
    p64.check()
    p64.close()
    p32.close()
    return err


def test_noncubic_config_against_oracle(torch_cuda):
    err = _against_oracle(torch_cuda, "noncubic", 1234)
    assert err["f64_forward_normalised_linf_vs_oracle"] <= 1e-12
    assert err["f64_backward_normalised_linf_vs_oracle"] <= 1e-12
    assert err["f64_roundtrip_max_abs"] <= err["roundtrip_rule_f64"]
    assert err["f64_roundtrip_normalised_linf"] <= 1e-12
    assert err["f32_forward_rel_l2_vs_oracle"] <= 1e-6
    assert err["f32_backward_rel_l2_vs_oracle"] <= 1e-6
    assert err["f32_roundtrip_max_abs"] <= err["roundtrip_rule_f32"]
    # the noise adds ~1e-3 sqrt(N) ~ 20 to modes of amplitude ~N/2 ~ 1e8
    assert err["modes_checked"] >= 30 and err["f64_modes_max_rel_err"] <= 1e-5


def test_chebyshev_config_against_oracle(torch_cuda):
    err = _against_oracle(torch_cuda, "cheby", 77)
    assert err["f64_forward_normalised_linf_vs_oracle"] <= 1e-12
    assert err["f64_backward_normalised_linf_vs_oracle"] <= 1e-12
    assert err["f64_roundtrip_normalised_linf"] <= 1e-12
    assert err["f64_cheby_normalised_linf_vs_oracle"] <= 1e-12
    assert err["f32_forward_rel_l2_vs_oracle"] <= 1e-6
    assert err["f32_backward_rel_l2_vs_oracle"] <= 1e-6
