"""Admission order of the serving loop (p3dfft_gb300.serve.Server._select),
checked on the host: FIFO without a work bound; with one, least estimated
work first up to the bound (at least one request), requests past the age
limit first, and the device-memory budget respected.  No GPU: the server
object is built without its CUDA streams and with a fixed byte count per
request."""
import collections

import pytest

serve = pytest.importorskip("p3dfft_gb300.serve")


def _server(launch_work, age_limit=0.008, budget=10**12, max_jobs=64, nbytes=1, now=0.0):
    srv = serve.Server.__new__(serve.Server)
    srv.pending = collections.deque()
    srv.max_jobs = max_jobs
    srv.launch_work = launch_work
    srv.age_limit = age_limit
    srv.budget = budget
    srv.in_flight_bytes = 0
    srv.request_bytes = lambda r: nbytes
    srv.now = lambda: now
    return srv


def _req(rid, side, arrival=0.0, kind="forward", tol=serve.F32_TOL):
    r = serve.Request(rid=rid, kind=kind, shape=(side, side, side), arrival=arrival, tol=tol)
    r.precision = serve.F64 if tol < serve.F32_TOL else serve.F32
    return r


def test_fifo_without_work_bound():
    srv = _server(None, max_jobs=3, now=0.001)
    for i, s in enumerate([256, 32, 64, 48]):
        srv.pending.append(_req(i, s))
    assert [r.rid for r in srv._select(0)] == [0, 1, 2]
    assert [r.rid for r in srv.pending] == [3]


def test_least_work_first_up_to_the_bound():
    srv = _server(launch_work=2 * 64**3, now=0.001)
    for i, s in enumerate([256, 64, 32, 64, 48]):
        srv.pending.append(_req(i, s))
    took = [r.rid for r in srv._select(0)]
    assert took == [2, 4, 1]  # 32^3 + 48^3 + 64^3 fit the bound, the second 64^3 does not
    assert [r.rid for r in srv.pending] == [0, 3]


def test_one_request_even_above_the_bound():
    srv = _server(launch_work=10.0, now=0.001)
    srv.pending.append(_req(0, 512))
    srv.pending.append(_req(1, 512))
    assert [r.rid for r in srv._select(1)] == [0]


def test_aged_requests_go_first_and_fp64_counts_more():
    srv = _server(launch_work=3 * 100**3, age_limit=0.005, now=0.010)
    srv.pending.append(_req(0, 100, arrival=0.0))                 # waited 10 ms: first
    srv.pending.append(_req(1, 80, arrival=0.009, tol=1e-12))     # FP64: 2.5 x 80^3
    srv.pending.append(_req(2, 90, arrival=0.009))
    took = [r.rid for r in srv._select(0)]
    assert took[0] == 0
    assert took == [0, 2]  # 100^3 + 90^3 fit, adding 2.5 x 80^3 would pass the bound
    assert serve.Server.work(_req(3, 10, kind="spectrum")) == pytest.approx(1.3 * 1000)


def test_budget_limits_admission():
    srv = _server(launch_work=1e12, budget=3, nbytes=2, now=0.001)
    for i in range(3):
        srv.pending.append(_req(i, 32))
    assert len(srv._select(0)) == 1
    assert srv.in_flight_bytes == 2
    srv2 = _server(launch_work=1e12, budget=1, nbytes=2, now=0.001)
    srv2.pending.append(_req(0, 32))
    with pytest.raises(RuntimeError, match="budget"):
        srv2._select(0)


def test_cancel_pending_request_on_the_host():
    srv = _server(launch_work=1e12, now=0.002)
    srv.slots = []
    srv.done = []
    for i, s in enumerate([32, 48, 64]):
        srv.pending.append(_req(i, s))
    assert srv.cancel(1) is True
    assert [r.rid for r in srv.pending] == [0, 2]
    assert srv.done[0].rid == 1 and srv.done[0].status == "cancelled" and srv.done[0].t_done == 0.002
    assert srv.cancel(7) is False
    took = srv._select(0)
    assert [r.rid for r in took] == [0, 2]


def test_summary_reports_the_slowest_requests():
    # summarize: percentiles over every request, and for the slowest 1 % the
    # mean time queued (arrival to admission) against in flight
    reqs = []
    for i in range(200):
        r = _req(i, 32, arrival=0.0)
        r.t_admit = 0.001
        r.t_done = 0.002 if i < 198 else 0.101  # two slow requests
        reqs.append(r)
    out = serve.summarize(reqs, wall_s=1.0)
    assert out["requests"] == 200 and out["throughput_req_s"] == 200.0
    assert out["p50_ms"] == pytest.approx(2.0)
    tail = out["p99_tail"]
    assert tail["requests"] == 2
    assert tail["queued_ms"] == pytest.approx(1.0)
    assert tail["in_flight_ms"] == pytest.approx(100.0)
