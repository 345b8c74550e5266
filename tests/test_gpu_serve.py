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


@pytest.mark.parametrize("host_direct", [True, False])
def test_serve_requests_with_their_own_host_data(torch_cuda, host_direct):
    # each request's input comes from host memory of its own (real inputs
    # read by the kernel over the host link, or every input copied to the
    # device first) and its result is copied back: the host results match
    # the oracle
    from p3dfft_gb300 import serve
    reqs = serve.attach_host_data(_small_requests(16, seed=14), seed=3, arena_bytes=64 << 20)
    srv = serve.Server(budget_bytes=8e9, slots=2, max_jobs=6, host_direct=host_direct)
    srv.run(reqs)
    for r in reqs:
        assert r.status == "done"
        r.inp = r.host_in
        r.out = r.host_out
        _oracle_check(r)
    srv.close()


def test_serve_requests_with_their_own_device_data(torch_cuda):
    # each request transforms its own view of a device arena (the bench's
    # device-data run): the results match the oracle
    from p3dfft_gb300 import serve
    reqs = serve.attach_device_data(_small_requests(16, seed=15), seed=4, arena_bytes=64 << 20)
    inputs = [r.inp.clone() for r in reqs]
    srv = serve.Server(budget_bytes=8e9, slots=2, max_jobs=6)
    srv.run(reqs)
    for r, x in zip(reqs, inputs):
        assert r.status == "done"
        r.inp = x
        _oracle_check(r)
    srv.close()


def test_serve_allocation_failure_fails_only_its_request(torch_cuda):
    # failure injected on the host: the work buffer of every fourth request
    # fails to allocate; the others complete and the budget is freed
    from p3dfft_gb300 import serve
    torch = torch_cuda
    reqs = _small_requests(12, seed=15)
    victims = {r.rid for r in reqs[::4]}
    srv = serve.Server(budget_bytes=8e9, slots=2, max_jobs=4)
    real_alloc = srv.alloc
    current = {}

    def alloc(shape, dtype):
        if current.get("rid") in victims:
            raise RuntimeError("CUDA out of memory (injected)")
        return real_alloc(shape, dtype)

    def job(r, inp, _orig=srv._job):
        current["rid"] = r.rid
        return _orig(r, inp)

    srv.alloc = alloc
    srv._job = job
    srv.run(reqs)
    for r in reqs:
        if r.rid in victims:
            assert r.status == "failed" and "injected" in r.error and r.out is None
        else:
            assert r.status == "done"
            _oracle_check(r)
    assert srv.in_flight_bytes == 0
    srv.close()
    del torch


def test_serve_cancellation(torch_cuda):
    from p3dfft_gb300 import serve
    reqs = _small_requests(10, seed=16)
    srv = serve.Server(budget_bytes=8e9, slots=1, max_jobs=2, launch_work=None)
    for r in reqs:
        srv.submit(r)
    assert srv.cancel(reqs[9].rid)           # pending: leaves the queue
    srv.poll()                               # launches the first two
    assert srv.cancel(reqs[0].rid)           # in flight: result discarded at retire
    srv.drain()
    assert reqs[9].status == "cancelled" and reqs[0].status == "cancelled" and reqs[0].out is None
    for r in reqs[1:9]:
        assert r.status == "done"
        _oracle_check(r)
    assert srv.in_flight_bytes == 0
    srv.close()


def test_serve_fp64_fallbacks(torch_cuda):
    # an FP32 request whose sums pass binary32's range is computed again on
    # the FP64 path; an FP64 request beyond the double-float window is
    # computed again with the bias picked on the device
    import torch as _t

    from p3dfft_gb300 import F64, serve
    big32 = serve.Request(rid=0, kind="forward", shape=(32, 32, 32),
                          host_in=_t.full((32, 32, 32), 3e37, dtype=_t.float32).pin_memory())
    rng = np.random.default_rng(17)
    big64 = serve.Request(rid=1, kind="backward", shape=(24, 20, 18), tol=1e-12,
                          host_in=_t.from_numpy(rng.standard_normal((18, 20, 13)) * 1e200
                                                + 1j * rng.standard_normal((18, 20, 13)) * 1e200).pin_memory())
    small = serve.Request(rid=2, kind="forward", shape=(16, 16, 16),
                          host_in=_t.from_numpy(rng.uniform(-1, 1, (16, 16, 16)).astype(np.float32)).pin_memory())
    srv = serve.Server(budget_bytes=8e9, slots=1, max_jobs=4)
    srv.run([big32, big64, small])
    assert big32.fallback and big32.precision == F64 and bool(_t.isfinite(big32.out).all())
    assert big64.fallback and small.status == "done" and not small.fallback
    for r in (big32, big64, small):
        r.inp = r.host_in
        _oracle_check(r)
    srv.close()
