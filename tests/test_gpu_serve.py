"""Serving form (p3dfft_gb300.serve): continuous batching over the batch
kernel.  Each request's result must be the same alone and in the mix --
bit for bit for transforms (same kernels and arithmetic), within binary64
rounding (normalised L-inf 1e-12) for spectra, whose shell sums are added
in a run-dependent order -- and match the oracle (F64 normalised L-inf
1e-12, F32 relative L2 1e-6)."""
import numpy as np
import pytest

from oracle import p3dfft_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import p3dfft_gb300  # noqa: F401
    return torch


def _small_requests(n, seed):
    from p3dfft_gb300 import serve
    return serve.make_requests(n, seed=seed, lo=16, hi=64, f64_fraction=0.3)


def _alone(torch, r):
    """The request run by itself through a one-job server."""
    from p3dfft_gb300 import serve
    one = serve.Server(budget_bytes=8e9, slots=1, max_jobs=1)
    q = serve.Request(rid=r.rid, kind=r.kind, shape=r.shape, tol=r.tol, inp=r.inp)
    one.run([q])
    out = q.out.clone()
    one.close()
    return out


def _oracle_check(r):
    from p3dfft_gb300 import F64
    nx, ny, nz = r.shape
    ref = orc.OraclePlan(nx, ny, nz)
    a = r.inp.cpu().numpy().astype(np.complex128 if r.kind == "backward" else np.float64)
    got = r.out.cpu().numpy()
    if r.kind == "forward":
        want = ref.ftran_r2c(a)
    elif r.kind == "backward":
        want = ref.btran_c2r(a)
    else:
        b = ref.ftran_r2c(a) / (nx * ny * nz)
        want = orc.shell_spectrum(b, nx, ny, nz, k2_weight=False, hermitian=True)
    if r.precision == F64 or r.kind == "spectrum":
        tol = 1e-12 if r.precision == F64 else 2e-6
        assert orc.normalised_linf(got, want) <= tol, (r.kind, r.shape)
    else:
        assert orc.relative_l2(got.astype(want.dtype), want) <= 1e-6, (r.kind, r.shape)


def test_serve_same_alone_and_in_mix(torch_cuda):
    from p3dfft_gb300 import serve
    torch = torch_cuda
    reqs = _small_requests(36, seed=11)
    srv = serve.Server(budget_bytes=8e9, slots=2, max_jobs=5)
    srv.run(reqs)  # all arrive at t = 0: several overlapping launches
    assert srv.launches >= 4 and max(srv.batch_sizes) <= 5
    for r in reqs:
        assert np.isfinite(r.latency) and r.latency >= 0
        alone = _alone(torch, r)
        if r.kind == "spectrum":
            assert orc.normalised_linf(r.out.cpu().numpy(), alone.cpu().numpy()) <= 1e-12
        else:
            assert torch.equal(r.out, alone), (r.kind, r.shape, r.precision)
        _oracle_check(r)
    srv.close()


def test_serve_budget_admission(torch_cuda):
    from p3dfft_gb300 import serve
    reqs = _small_requests(12, seed=12)
    srv = serve.Server(budget_bytes=1, slots=2, max_jobs=8)  # nothing fits a 1-byte budget
    with pytest.raises(RuntimeError, match="budget"):
        srv.run(reqs)
    srv.close()
    # a budget of about two requests: launches stay small, everything completes
    srv = serve.Server(budget_bytes=1, slots=2, max_jobs=8)
    need = max(srv.request_bytes(r) for r in reqs)
    srv.budget = 2 * need
    srv.resident_limit = 2 * need
    srv.run(reqs)
    assert all(np.isfinite(r.latency) for r in reqs)
    assert 0 < srv.peak_in_flight <= srv.budget
    for r in reqs:
        _oracle_check(r)
    srv.close()


def test_serve_poisson_stream_reports_latency(torch_cuda):
    from p3dfft_gb300 import serve
    reqs = serve.poisson_arrivals(_small_requests(40, seed=13), rate=2000.0)
    srv = serve.Server(budget_bytes=8e9, slots=3, max_jobs=16, keep_outputs=False)
    t = __import__("time").perf_counter()
    srv.run(reqs)
    wall = __import__("time").perf_counter() - t
    s = serve.summarize(reqs, wall)
    assert s["requests"] == 40 and 0 <= s["p50_ms"] <= s["p99_ms"]
    assert all(r.out is None for r in reqs)
    srv.close()
