"""The allocation-free forward transform (p3g_ftran_r2c_noalloc).

It exists for callers that cannot allocate device memory once running
(fixed-budget serving workers, frameworks owning every allocation, loops that
cannot take cudaMalloc's synchronisation); its workspace is a fixed device
array inside the library.  This file is collected last on purpose.  Each case
calls the entry point through the C ABI twice in a row and checks each result
against the allocating entry point p3g_ftran_r2c (F64: normalised L-inf
1e-12; F32: relative L2 1e-6) and against the CPU oracle, and a grid whose
workspace exceeds the fixed scratch is refused with a clear error.
"""
import ctypes

import numpy as np
import pytest

from oracle import p3dfft_oracle as orc

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-6
E_UNSUPPORTED = -4


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300
    from p3dfft_gb300 import _lib
    return torch, p3dfft_gb300, _lib.load().core


CASES = [
    # (grid and pruned sizes, op, precision, layout)
    ((64, 48, 40), "fft", "f64", 0),
    ((32, 30, 20, 32, 24, 20), "fft", "f64", 0),
    ((32, 16, 17), "ffc", "f64", 0),
    ((24, 20, 18), "ffs", "f64", 0),
    ((24, 20, 18), "ffn", "f64", 0),
    ((40, 24, 30), "fft", "f64", 1),
    ((64, 48, 40), "fft", "f32", 0),
    ((30, 36, 28, 30, 20, 28), "fft", "f32", 0),  # nyc < ny: wb after the 256-byte-rounded wa
    ((33, 30, 25), "ffc", "f32", 0),
    ((24, 20, 18), "ffs", "f32", 0),
    ((24, 20, 18), "ffn", "f32", 0),
]


@pytest.mark.parametrize("args,op,prec,layout", CASES)
def test_noalloc_matches_allocating_forward_and_oracle(cuda, args, op, prec, layout):
    torch, pg, core = cuda
    nx, ny, nz = args[:3]
    f64 = prec == "f64"
    plan = pg.Plan(*args, precision=pg.F64 if f64 else pg.F32, layout=layout)
    a = np.random.default_rng(31).uniform(-1, 1, size=(nz, ny, nx))
    x = torch.from_numpy(a).cuda()
    if not f64:
        x = x.float()
    want = plan.ftran_r2c(x, op=op).cpu().numpy()
    ref = orc.OraclePlan(*args, stride1=bool(layout)).ftran_r2c(a if f64 else x.double().cpu().numpy(), op)
    cdt = torch.complex128 if f64 else torch.complex64
    for _ in range(2):
        out = torch.full(plan.complex_shape, float("nan"), dtype=cdt, device="cuda")
        rc = core.p3g_ftran_r2c_noalloc(plan._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                        op.encode(), None)
        assert rc == 0, core.p3g_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        if f64:
            assert orc.normalised_linf(got, want) <= TOL64
            assert orc.normalised_linf(got, ref) <= TOL64
        else:
            assert orc.relative_l2(got.astype(np.complex128), want.astype(np.complex128)) <= TOL32
            assert orc.relative_l2(got.astype(np.complex128), ref) <= TOL32
    plan.close()


def test_noalloc_rejects_grids_beyond_its_scratch(cuda):
    torch, pg, core = cuda
    plan = pg.Plan(512, 512, 512)  # ~1.1 GB of workspace
    x = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = core.p3g_ftran_r2c_noalloc(plan._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()), b"fft",
                                    None)
    assert rc == E_UNSUPPORTED
    assert b"scratch" in core.p3g_last_error()
    plan.close()
