"""The allocation-free forward transform (p3g_ftran_r2c_noalloc).

It exists for callers that cannot allocate device memory once running
(fixed-budget serving workers, frameworks owning every allocation, loops that
cannot take cudaMalloc's synchronisation); its workspace is a fixed device
array inside the library.  This file is collected last on purpose.  The
test calls the entry point through the C ABI twice in a row and checks each
result against the allocating entry point p3g_ftran_r2c, to the F64 parity
tolerance (normalised L-inf 1e-12), and checks that a grid whose workspace
exceeds the fixed scratch is refused with a clear error.
"""
import ctypes

import numpy as np
import pytest

from oracle import p3dfft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-12
E_UNSUPPORTED = -4


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300
    from p3dfft_gb300 import _lib
    return torch, p3dfft_gb300, _lib.load().core


@pytest.mark.parametrize("args,op", [((64, 48, 40), "fft"), ((32, 30, 20, 32, 24, 20), "fft"),
                                     ((32, 16, 17), "ffc")])
def test_noalloc_matches_allocating_forward(cuda, args, op):
    torch, pg, core = cuda
    nx, ny, nz = args[:3]
    plan = pg.Plan(*args)
    a = np.random.default_rng(31).uniform(-1, 1, size=(nz, ny, nx))
    x = torch.from_numpy(a).cuda()
    want = plan.ftran_r2c(x, op=op).cpu().numpy()
    for _ in range(2):
        out = torch.full(plan.complex_shape, float("nan"), dtype=torch.complex128, device="cuda")
        rc = core.p3g_ftran_r2c_noalloc(plan._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                        op.encode(), None)
        assert rc == 0, core.p3g_last_error()
        torch.cuda.synchronize()
        assert orc.normalised_linf(out.cpu().numpy(), want) <= TOL
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
