"""The sm_103a transforms against the committed closed-form fixtures
(tests/golden), F64 path (normalised L-inf 1e-12), through the explicit API
and through the drop-in library."""
import numpy as np
import pytest

import golden_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300  # noqa: F401
    return torch


def test_plan_matches_golden_fixtures(torch_cuda):
    import p3dfft_gb300 as pg
    torch = torch_cuda

    class _Gpu:
        def __init__(self, nx, ny, nz):
            self.p = pg.Plan(nx, ny, nz, precision=pg.F64)

        def ftran(self, a, op):
            return self.p.ftran_r2c(torch.from_numpy(np.ascontiguousarray(a)).cuda(), op=op).cpu().numpy()

        def btran(self, c, op):
            return self.p.btran_c2r(torch.from_numpy(np.ascontiguousarray(c)).cuda(), op=op).cpu().numpy()

        def cheby(self, a, lz):
            return self.p.cheby(torch.from_numpy(np.ascontiguousarray(a)).cuda(), lz).cpu().numpy()

    golden_cases.check_all(_Gpu, 1e-12)


def test_drop_in_matches_golden_fixtures(torch_cuda):
    import p3dfft_gb300 as pg

    class _DropIn:
        def __init__(self, nx, ny, nz):
            self.shape = (nx, ny, nz)

        def _run(self, fn, src, shape, dtype, *extra):
            nx, ny, nz = self.shape
            pg.p3dfft_setup((1, 1), nx, ny, nz)
            try:
                out = np.zeros(shape, dtype=dtype)
                fn(np.ascontiguousarray(src), out, *extra)
            finally:
                pg.p3dfft_clean()
            return out

        def ftran(self, a, op):
            nx, ny, nz = self.shape
            return self._run(pg.p3dfft_ftran_r2c, a, (nz, ny, nx // 2 + 1), np.complex128, op)

        def btran(self, c, op):
            nx, ny, nz = self.shape
            return self._run(pg.p3dfft_btran_c2r, c.astype(np.complex128), (nz, ny, nx), np.float64, op)

        def cheby(self, a, lz):
            nx, ny, nz = self.shape
            return self._run(pg.p3dfft_cheby, a, (nz, ny, nx // 2 + 1), np.complex128, lz)

    golden_cases.check_all(_DropIn, 1e-12)
