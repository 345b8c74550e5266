"""Serving form: a request loop with continuous batching.

Requests are forward r2c transforms, backward c2r transforms, or power
spectra (forward transform, then |u_hat|^2 binned into integer spherical
shells in binary64 with the conjugate half counted), of any grid size.
Plans (twiddles, stage tables) and each shape's input grid stay resident on
the device.  The loop keeps ``slots`` launch slots, each a CUDA stream with
one batch object per precision; whenever a slot is free it admits pending
requests that fit the device-memory budget and the per-launch job limit,
and launches them as one persistent batch (p3g_batch_*) per precision.
Requests that arrive while other slots are busy are admitted as slots and
memory free up, and the slots' launches overlap on the GPU.

Scheduling (``launch_work``; None = FIFO): a free slot takes the pending
requests with the least estimated work first (points x 2.5 for FP64, x 1.3
for spectra) until the launch holds ``launch_work`` point-equivalents (at
least one request), except that a request that has waited ``age_limit``
seconds goes first.  Every result of a launch is known only when the whole
launch ends, so bounded launches keep a small request from waiting for a
large batch; the size order keeps bursts of small requests from queueing
behind large ones, and the age limit keeps large requests from starving.
Measured at 70 % load (10,000 requests of sides 32..512, each with its own
device input): p99 10.5 ms with a 20M-point bound against 12.1 ms with 40M
(8 % more closed-loop capacity) and ~77 ms with 40M and a 4 ms age limit;
FIFO admission had given p99 22 ms against 16 ms with a 40M bound.

Admission: a request holds its input, output and work buffer while in
flight, and the sum over in-flight requests stays within the device-memory
budget (a request larger than the whole budget is an error).  Resident
input grids are kept besides, up to a quarter of the budget, least recently
used first out.

Precision per request: the FP32 path (compensated twiddles; relative L2
error ~2e-7 against the FP64 oracle) unless the request asks for a tighter
tolerance than ``F32_TOL``, then the FP64 path (double-float; ~1e-14).
Fallback at run time: an FP32 result that is not finite (a field beyond
binary32's range) is computed again on the FP64 path, and an FP64 batch
whose inputs left the double-float exponent window (p3g_batch_status
reports P3G_E_RANGE) has its FP64 requests computed again through the plain
API with the exponent bias picked on the device; ``Request.fallback``
records it.

Request data: a request either names a device tensor (``inp``), or brings
host memory (``host_in``, page-locked): a real input (forward, spectrum) is
read by the batch kernel's X pass over the host link directly
(``host_direct``), a complex one (backward, whose Z pass reads strided runs
that cross the link slowly) is copied to a device buffer of its own on the
slot's stream just before its launch; with ``host_out`` the result is copied
back on the same stream, so the request's latency includes its own data
movement.  Without either the
request uses the shape's resident input grid.

Failures stay per request: a device buffer that cannot be allocated fails
only its request (``status`` "failed", ``error`` the message) and frees its
share of the budget; ``cancel(rid)`` drops a pending request at once and
discards an in-flight one's result when its launch retires.  ``alloc`` is
the one place buffers come from, so a test can make it fail on the host.

There is no counterpart in the reference (one blocking transform per call);
the transforms themselves are the reference's (ftran.F90:489-780,
btran.F90:396-679) and the spectrum is the spectrum sample's binning
(driver_spec.F90:263-341).
"""
from __future__ import annotations

import collections
import math
import time
from dataclasses import dataclass, field

from . import (F32, F64, JOB_BACKWARD, JOB_FORWARD, JOB_SPECTRUM, SPEC_HERMITIAN, Batch, Plan)

F32_TOL = 1e-6
KINDS = {"forward": JOB_FORWARD, "backward": JOB_BACKWARD, "spectrum": JOB_SPECTRUM}


@dataclass
class Request:
    rid: int
    kind: str                 # forward | backward | spectrum
    shape: tuple              # (nx, ny, nz)
    arrival: float = 0.0      # seconds on the server's clock
    tol: float = F32_TOL      # requested accuracy; < F32_TOL selects FP64
    precision: int = F32
    t_admit: float = math.nan
    t_done: float = math.nan
    out: object = None        # result tensor
    inp: object = None        # input tensor (resident per shape unless given)
    host_in: object = None    # host input copied to a device buffer of its own
    host_out: object = None   # host tensor the result is copied back to
    nbytes: int = 0           # device bytes held while in flight
    slot: int = -1
    status: str = "pending"   # pending, done, cancelled, failed
    error: str = ""
    cancelled: bool = False
    fallback: bool = False    # computed again on the FP64 path
    resident: bool = False    # inp is the shape's resident grid (counted in use)

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival

    @property
    def points(self) -> int:
        return self.shape[0] * self.shape[1] * self.shape[2]


def kmax_of(shape) -> int:
    nx, ny, nz = shape
    return int(math.sqrt(float(nx) * nx + ny * ny + nz * nz) * 0.5 + 0.5)


@dataclass
class _Slot:
    stream: object
    batches: dict
    event: object = None
    reqs: list = field(default_factory=list)
    busy: bool = False
    finite: object = None  # per FP32 request of the launch: result finite
    # page-locked copy of `finite`, written on the slot's stream before its
    # event: read at retire without a synchronous copy (which would queue
    # behind other slots' bulk copies on the copy engines)
    finite_host: object = None


class Server:
    """Continuous-batching transform server on the current CUDA device."""

    def __init__(self, budget_bytes: float = 150e9, slots: int = 3, max_jobs: int = 64, window: int = 4,
                 tuned: bool = False, keep_outputs: bool = True, launch_work: float = 20e6,
                 age_limit: float = 0.008, host_direct: bool = True):
        import torch
        self.torch = torch
        self.budget = int(budget_bytes)
        self.max_jobs = max_jobs
        self.launch_work = launch_work
        self.age_limit = age_limit
        self.host_direct = host_direct
        self.window = window
        self.tuned = tuned
        self.keep_outputs = keep_outputs
        self.plans = {}
        # resident input grids, least recently used first; bounded by a
        # quarter of the budget (grids in use by in-flight requests stay)
        self.resident = collections.OrderedDict()   # (shape, precision, backward) -> tensor
        self.resident_limit = self.budget // 4
        self.in_use = collections.Counter()
        self.resident_bytes = 0
        self.in_flight_bytes = 0
        self.peak_bytes = 0
        self.peak_in_flight = 0
        self.pending = collections.deque()
        self.done = []
        self.launches = 0
        self.batch_sizes = []
        self.slots = [_Slot(stream=torch.cuda.Stream(), batches={F32: Batch(F32), F64: Batch(F64)})
                      for _ in range(slots)]
        self.t0 = time.perf_counter()

    # ------------------------------------------------------------ resources
    def now(self) -> float:
        return time.perf_counter() - self.t0

    def plan(self, shape, precision) -> Plan:
        key = (tuple(shape), precision)
        p = self.plans.get(key)
        if p is None:
            if self.tuned:
                from .autotune import tuned_plan
                p = tuned_plan(tuple(shape), precision)
            else:
                p = Plan(*shape, precision=precision)
            self.plans[key] = p
        return p

    def _dtypes(self, precision):
        t = self.torch
        return (t.float64, t.complex128) if precision == F64 else (t.float32, t.complex64)

    def _input_key(self, req: Request):
        return (tuple(req.shape), req.precision, req.kind == "backward")

    def resident_input(self, shape, precision, kind, seed=0):
        """The shape's input grid, created once on the device: U[-1,1) reals,
        or for backward requests a complex N(0,1) spectrum."""
        key = (tuple(shape), precision, kind == "backward")
        x = self.resident.get(key)
        if x is not None:
            self.resident.move_to_end(key)
            return x
        t = self.torch
        nx, ny, nz = shape
        rdt, cdt = self._dtypes(precision)
        g = t.Generator(device="cuda")
        g.manual_seed(hash((tuple(shape), seed)) & 0x7FFFFFFF)
        if kind == "backward":
            x = t.randn((nz, ny, nx // 2 + 1), generator=g, device="cuda", dtype=cdt)
        else:
            x = t.rand((nz, ny, nx), generator=g, device="cuda", dtype=t.float64).mul_(2).sub_(1).to(rdt)
        self.resident[key] = x
        self.resident_bytes += x.numel() * x.element_size()
        for k in list(self.resident):
            if self.resident_bytes <= self.resident_limit or k == key:
                break
            if self.in_use[k] == 0:
                old = self.resident.pop(k)
                self.resident_bytes -= old.numel() * old.element_size()
        return x

    def request_bytes(self, req: Request) -> int:
        """Device bytes a request holds while in flight: its input grid, its
        output and its batch work buffer."""
        p = self.plan(req.shape, req.precision)
        nx, ny, nz = req.shape
        rsz = 8 if req.precision == F64 else 4
        real = nx * ny * nz * rsz
        cplx = (nx // 2 + 1) * ny * nz * 2 * rsz
        if req.kind == "forward":
            io = real + cplx
        elif req.kind == "backward":
            io = cplx + real
        else:
            io = real + (kmax_of(req.shape) + 1) * 8
        return io + p.work_bytes(KINDS[req.kind])

    @staticmethod
    def work(req: Request) -> float:
        """Estimated work of a request in point-equivalents."""
        w = float(req.points)
        if req.precision == F64:
            w *= 2.5
        if req.kind == "spectrum":
            w *= 1.3
        return w

    def _admit(self, req: Request, slot_index: int) -> bool:
        """Reserves the request's device bytes; False when they do not fit now."""
        nb = self.request_bytes(req)
        if nb > self.budget:
            raise RuntimeError(f"request {req.rid} needs {nb} device bytes, above the device-memory "
                               f"budget of {self.budget}")
        if self.in_flight_bytes + nb > self.budget:
            return False
        req.nbytes = nb
        req.t_admit = self.now()
        req.slot = slot_index
        self.in_flight_bytes += nb
        return True

    def _select(self, slot_index: int):
        """The requests of the next launch (removed from the queue)."""
        take = []
        if self.launch_work is None:  # FIFO
            while self.pending and len(take) < self.max_jobs:
                if not self._admit(self.pending[0], slot_index):
                    break
                take.append(self.pending.popleft())
            return take
        now = self.now()
        order = sorted(self.pending, key=self.work)
        old = [r for r in self.pending if now - r.arrival >= self.age_limit]
        if old:  # oldest first, then by size
            order = old + [r for r in order if now - r.arrival < self.age_limit]
        total = 0.0
        chosen = set()  # ids of the chosen requests
        for r in order:
            if len(take) >= self.max_jobs:
                break
            w = self.work(r)
            if take and total + w > self.launch_work:
                break
            if not self._admit(r, slot_index):
                break
            take.append(r)
            chosen.add(id(r))
            total += w
        if chosen:
            self.pending = collections.deque(r for r in self.pending if id(r) not in chosen)
        return take

    def alloc(self, shape, dtype):
        """Every device buffer of a request comes from here (a test replaces
        it to make allocations fail)."""
        return self.torch.empty(shape, dtype=dtype, device="cuda")

    # ------------------------------------------------------------ the loop
    def submit(self, req: Request) -> None:
        req.precision = F64 if req.tol < F32_TOL else F32
        req.status = "pending"
        self.pending.append(req)

    def cancel(self, rid: int) -> bool:
        """Cancels request rid: a pending one leaves the queue now, an
        in-flight one's result is discarded when its launch retires.  False
        when no such request is pending or in flight."""
        for r in self.pending:
            if r.rid == rid:
                self.pending.remove(r)
                r.cancelled = True
                r.status = "cancelled"
                r.t_done = self.now()
                self.done.append(r)
                return True
        for s in self.slots:
            for r in s.reqs:
                if r.rid == rid:
                    r.cancelled = True
                    return True
        return False

    def _release(self, r: Request) -> None:
        self.in_flight_bytes -= r.nbytes
        if r.resident:
            key = self._input_key(r)
            if self.in_use[key] > 0:
                self.in_use[key] -= 1
            r.resident = False

    def _fail(self, r: Request, err: Exception) -> None:
        r.status = "failed"
        r.error = str(err)
        r.t_done = self.now()
        r.out = None
        r.inp = None
        self._release(r)
        self.done.append(r)

    def _job(self, r: Request, inp):
        """Output buffer and batch job of a request (allocations through alloc)."""
        t = self.torch
        p = self.plan(r.shape, r.precision)
        rdt, cdt = self._dtypes(r.precision)
        nx, ny, nz = r.shape
        work = self.alloc(p.work_bytes(KINDS[r.kind]), t.uint8)
        if r.kind == "forward":
            r.out = self.alloc(p.complex_shape, cdt)
            return {"plan": p, "kind": JOB_FORWARD, "in": inp, "out": r.out, "work": work}
        if r.kind == "backward":
            r.out = self.alloc((nz, ny, nx), rdt)
            return {"plan": p, "kind": JOB_BACKWARD, "in": inp, "out": r.out, "work": work}
        r.out = self.alloc(kmax_of(r.shape) + 1, t.float64)
        return {"plan": p, "kind": JOB_SPECTRUM, "in": inp, "out": r.out, "work": work,
                "kmax": kmax_of(r.shape), "scale": 1.0 / (nx * ny * nz), "flags": SPEC_HERMITIAN}

    def _launch(self, slot: _Slot, reqs) -> None:
        t = self.torch
        groups = {F32: [], F64: []}
        live, copies = [], []
        for r in reqs:
            try:
                rdt, cdt = self._dtypes(r.precision)
                if (r.host_in is not None and self.host_direct and r.kind != "backward" and
                        r.host_in.dtype == rdt and r.host_in.is_contiguous() and r.host_in.is_pinned()):
                    # a real input in page-locked memory: the X pass reads its
                    # lines over the host link itself, with no copy queued on
                    # the copy engines behind other launches' bulk copies
                    r.inp = r.host_in
                elif r.host_in is not None:
                    # the request's own data: a device buffer filled on the slot's stream
                    r.inp = self.alloc(tuple(r.host_in.shape), cdt if r.kind == "backward" else rdt)
                    copies.append((r.inp, r.host_in))
                elif r.inp is None:
                    r.inp = self.resident_input(r.shape, r.precision, r.kind)
                    r.resident = True
                    self.in_use[self._input_key(r)] += 1
                job = self._job(r, r.inp)
            except (RuntimeError, MemoryError) as e:  # torch's out-of-memory error is a RuntimeError
                self._fail(r, e)
                continue
            groups[r.precision].append(job)
            live.append(r)
        # the slot's launch follows everything queued on the current stream
        # (input grids generated there, allocations of the buffers above)
        slot.stream.wait_stream(t.cuda.current_stream())
        with t.cuda.stream(slot.stream):
            for dev, host in copies:
                dev.copy_(host.to(dev.dtype) if host.dtype != dev.dtype else host, non_blocking=True)
            for prec, jobs in groups.items():
                if jobs:
                    b = slot.batches[prec]
                    b.set_jobs(jobs, window=self.window)
                    b.launch(slot.stream)
                    self.launches += 1
            # finiteness of the FP32 results (read at retire, no extra wait) and
            # the copies back to the host
            f32 = [r for r in live if r.precision == F32]
            slot.finite = t.stack([t.isfinite(r.out).all() for r in f32]) if f32 else None
            if f32:
                if slot.finite_host is None or slot.finite_host.numel() < len(f32):
                    slot.finite_host = t.empty(max(len(f32), self.max_jobs), dtype=t.bool).pin_memory()
                slot.finite_host[:len(f32)].copy_(slot.finite, non_blocking=True)
            for r in live:
                if r.host_out is not None:
                    r.host_out.copy_(r.out, non_blocking=True)
            slot.event = t.cuda.Event()
            slot.event.record(slot.stream)
        slot.reqs = live
        slot.busy = True
        self.batch_sizes.append(len(live))


    def _rerun(self, r: Request, precision) -> None:
        """Computes r again through the plain API on `precision` (FP64 with the
        exponent bias picked on the device) on the current stream."""
        from . import RANGE_AUTO
        t = self.torch
        p = self.plan(r.shape, precision)
        rdt, cdt = self._dtypes(precision)
        src = r.host_in if r.host_in is not None else r.inp
        inp = src.to(device="cuda", dtype=cdt if r.kind == "backward" else rdt)
        nx, ny, nz = r.shape
        if precision == F64:
            p.set_range(RANGE_AUTO)
        try:
            if r.kind == "forward":
                r.out = p.ftran_r2c(inp)
            elif r.kind == "backward":
                r.out = p.btran_c2r(inp)
            else:
                b = p.ftran_r2c(inp)
                r.out = p.spectrum(b, kmax=kmax_of(r.shape), scale=1.0 / (nx * ny * nz), flags=SPEC_HERMITIAN)
            t.cuda.synchronize()
        finally:
            if precision == F64:
                p.set_range()
        r.precision = precision

    def _retire(self, slot: _Slot) -> None:
        from . import P3DFFTError
        for prec, b in slot.batches.items():
            if any(r.precision == prec for r in slot.reqs):
                try:
                    b.check(slot.stream)
                except P3DFFTError as e:
                    if prec != F64 or "exponent window" not in str(e):
                        raise
                    for r in slot.reqs:  # FP64 inputs outside the window: again, biased
                        if r.precision == F64 and not r.cancelled:
                            r.fallback = True
                            self._rerun(r, F64)
            b._keep = []  # release the work buffers
        finite = slot.finite_host[:slot.finite.numel()].tolist() if slot.finite is not None else []
        i32 = 0
        for r in slot.reqs:
            ok = True
            if r.precision == F32:
                ok = bool(finite[i32])
                i32 += 1
            if r.cancelled:
                r.status = "cancelled"
                r.out = None
            else:
                if not ok:  # an FP32 result beyond binary32's range: FP64 fallback
                    r.fallback = True
                    self._rerun(r, F64)
                    if r.host_out is not None:
                        r.host_out = r.out.cpu()
                r.status = "done"
            r.t_done = self.now()
            self._release(r)
            if not self.keep_outputs:
                r.out = None
                r.inp = None
            self.done.append(r)
        slot.reqs = []
        slot.finite = None
        slot.busy = False

    def poll(self) -> bool:
        """Retire finished slots, then fill free slots from the queue.
        Returns True when something happened."""
        acted = False
        for s in self.slots:
            if s.busy and s.event.query():
                self._retire(s)
                acted = True
        for i, s in enumerate(self.slots):
            if s.busy or not self.pending:
                continue
            take = self._select(i)
            if not take:
                break
            self.peak_in_flight = max(self.peak_in_flight, self.in_flight_bytes)
            self.peak_bytes = max(self.peak_bytes, self.resident_bytes + self.in_flight_bytes)
            self._launch(s, take)
            acted = True
        return acted

    def drain(self) -> None:
        while self.pending or any(s.busy for s in self.slots):
            if not self.poll():
                time.sleep(20e-6)

    def run(self, requests):
        """Replays `requests` with their arrival times (seconds from the
        start of the call) and returns them completed (outputs dropped at
        completion unless the server keeps them)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        self.t0 = time.perf_counter()
        i = 0
        n = len(reqs)
        while i < n or self.pending or any(s.busy for s in self.slots):
            now = self.now()
            while i < n and reqs[i].arrival <= now:
                self.submit(reqs[i])
                i += 1
            if not self.poll():
                time.sleep(20e-6)
        return reqs

    def close(self) -> None:
        for s in self.slots:
            for b in s.batches.values():
                b.close()
        for p in self.plans.values():
            p.close()
        self.plans.clear()
        self.resident.clear()


# ------------------------------------------------------------------ workload
def smooth_sides(lo: int = 32, hi: int = 512):
    """All 2^a 3^b 5^c in [lo, hi]."""
    out = []
    a = 1
    while a <= hi:
        b = a
        while b <= hi:
            c = b
            while c <= hi:
                if c >= lo:
                    out.append(c)
                c *= 5
            b *= 3
        a *= 2
    return sorted(set(out))


def make_requests(n: int, seed: int = 5, lo: int = 32, hi: int = 512, mix=(4, 4, 2), f64_fraction: float = 0.1):
    """n requests: kinds forward:backward:spectrum = mix, cubic or box grids
    with sides log-uniform over the 2^a 3^b 5^c values in [lo, hi], and a
    fraction asking for FP64 accuracy.  Arrival times are filled in by
    poisson_arrivals."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sides = np.array(smooth_sides(lo, hi))
    logs = np.log(sides)
    kinds = np.array(["forward", "backward", "spectrum"])
    p = np.array(mix, dtype=float) / sum(mix)

    def side():
        u = rng.uniform(math.log(lo), math.log(hi))
        return int(sides[np.argmin(np.abs(logs - u))])

    reqs = []
    for i in range(n):
        if rng.random() < 0.5:
            s = side()
            shape = (s, s, s)
        else:
            shape = (side(), side(), side())
        kind = str(rng.choice(kinds, p=p))
        tol = 1e-12 if rng.random() < f64_fraction else F32_TOL
        reqs.append(Request(rid=i, kind=kind, shape=shape, tol=tol))
    return reqs


def attach_host_data(reqs, seed: int = 7, outputs: bool = True, arena_bytes: int = 1 << 30):
    """Gives every request host data of its own: an input view of a
    page-locked arena (real field, or complex spectrum for backward
    requests, in the request's precision) and, with outputs, a view of a
    second arena for its result.  Views rotate through the arenas, so the
    bytes repeat but each request's copies are its own."""
    import numpy as np
    import torch
    arena_in = torch.empty(arena_bytes, dtype=torch.uint8).pin_memory()
    rng = np.random.default_rng(seed)
    arena_in.view(torch.float32)[:] = torch.from_numpy(rng.uniform(-1, 1, arena_bytes // 4).astype(np.float32))
    arena_out = torch.empty(arena_bytes, dtype=torch.uint8).pin_memory() if outputs else None
    off_in = off_out = 0

    def take(arena, off, n):
        if off + n > arena_bytes:
            off = 0
        return arena[off:off + n], (off + n + 255) // 256 * 256

    for r in reqs:
        nx, ny, nz = r.shape
        f64 = r.tol < F32_TOL
        rdt = torch.float64 if f64 else torch.float32
        cdt = torch.complex128 if f64 else torch.complex64
        if r.kind == "backward":
            shape_in, dt_in = (nz, ny, nx // 2 + 1), cdt
        else:
            shape_in, dt_in = (nz, ny, nx), rdt
        n_in = int(np.prod(shape_in)) * dt_in.itemsize
        v, off_in = take(arena_in, off_in, n_in)
        r.host_in = v.view(dt_in).view(shape_in)
        if outputs:
            if r.kind == "forward":
                shape_out, dt_out = (nz, ny, nx // 2 + 1), cdt
            elif r.kind == "backward":
                shape_out, dt_out = (nz, ny, nx), rdt
            else:
                shape_out, dt_out = (kmax_of(r.shape) + 1,), torch.float64
            n_out = int(np.prod(shape_out)) * dt_out.itemsize
            v, off_out = take(arena_out, off_out, n_out)
            r.host_out = v.view(dt_out).view(shape_out)
    return reqs


def poisson_arrivals(reqs, rate: float, seed: int = 6):
    """Exponential inter-arrival times at `rate` requests per second."""
    import numpy as np
    rng = np.random.default_rng(seed)
    t = 0.0
    for r in reqs:
        t += rng.exponential(1.0 / rate)
        r.arrival = t
    return reqs


def attach_device_data(reqs, seed: int = 8, arena_bytes: int = 8 << 30):
    """Gives every request an input of its own in device memory: a view of a
    device arena of uniform values in [-1, 1) (binary32 for FP32 requests,
    binary64, a quarter of the bytes, for FP64 ones; real fields, or complex
    spectra for backward requests), views rotating through the arena, so
    each request transforms its own buffer with no host transfer."""
    import numpy as np
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    n64 = arena_bytes // 4 // 8
    n32 = (arena_bytes - n64 * 8) // 4
    arenas = {False: torch.empty(n32, dtype=torch.float32, device="cuda").uniform_(-1, 1, generator=g),
              True: torch.empty(n64, dtype=torch.float64, device="cuda").uniform_(-1, 1, generator=g)}
    offs = {False: 0, True: 0}
    for r in reqs:
        nx, ny, nz = r.shape
        f64 = r.tol < F32_TOL
        a = arenas[f64]
        if r.kind == "backward":
            shape_in, dt_in = (nz, ny, nx // 2 + 1), torch.complex128 if f64 else torch.complex64
        else:
            shape_in, dt_in = (nz, ny, nx), torch.float64 if f64 else torch.float32
        n = int(np.prod(shape_in)) * (2 if dt_in.is_complex else 1)
        if n > a.numel():
            raise ValueError(f"request {r.rid} needs {n} elements, more than the device arena holds")
        if offs[f64] + n > a.numel():
            offs[f64] = 0
        r.inp = a[offs[f64]:offs[f64] + n].view(dt_in).view(shape_in)
        offs[f64] = (offs[f64] + n + 63) // 64 * 64
    return reqs


def summarize(reqs, wall_s: float) -> dict:
    import numpy as np
    lat = np.array([r.latency for r in reqs]) * 1e3
    pts = sum(r.points for r in reqs)
    out = {"requests": len(reqs), "p50_ms": round(float(np.percentile(lat, 50)), 3),
           "p99_ms": round(float(np.percentile(lat, 99)), 3), "mean_ms": round(float(lat.mean()), 3),
           "throughput_req_s": round(len(reqs) / wall_s, 1), "gpts_per_s": round(pts / wall_s / 1e9, 3),
           "wall_s": round(wall_s, 3), "f64_requests": sum(1 for r in reqs if r.precision == F64)}
    # the slowest 1 %: time queued (arrival to admission) against time in
    # flight (admission to completion), and what they were
    tail = [r for r, l in zip(reqs, lat) if l >= np.percentile(lat, 99)]
    if tail:
        out["p99_tail"] = {
            "requests": len(tail),
            "queued_ms": round(float(np.mean([r.t_admit - r.arrival for r in tail])) * 1e3, 3),
            "in_flight_ms": round(float(np.mean([r.t_done - r.t_admit for r in tail])) * 1e3, 3),
            "mean_points": int(np.mean([r.points for r in tail])),
            "f64_share": round(sum(1 for r in tail if r.precision == F64) / len(tail), 3)}
    return out
