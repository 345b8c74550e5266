"""GB300-native P3DFFT 3D transform path.

Two interfaces over the same sm_103a kernels:

* ``Plan`` -- the explicit device API (include/p3dfft_gb300.h): device
  tensors, CUDA streams, F64 or F32 path, many fields per call.
* ``p3dfft_setup`` / ``p3dfft_get_dims`` / ``p3dfft_ftran_r2c`` /
  ``p3dfft_btran_c2r`` / ``p3dfft_*_many`` / ``p3dfft_cheby`` /
  ``p3dfft_clean`` / ``get_timers`` / ``set_timers`` -- the reference's module
  interface (build/module.F90:178-186, include/p3dfft.h) through the drop-in
  library, with the same argument meaning: arrays are column-major
  (X fastest), i.e. numpy C-order arrays shaped (nz, ny, nx) for real fields
  and (nzc, nyc, nxc/2+1) for complex ones; host numpy arrays or CUDA
  tensors are accepted.  Errors raise ``P3DFFTError`` where the reference
  prints and aborts.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

__all__ = [
    "P3DFFTError", "Plan", "F64", "F32", "p3dfft_setup", "p3dfft_get_dims", "p3dfft_get_mpi_info",
    "p3dfft_ftran_r2c", "p3dfft_btran_c2r", "p3dfft_ftran_r2c_many", "p3dfft_btran_c2r_many",
    "p3dfft_ftran_r2c_1d",
    "p3dfft_cheby", "p3dfft_cheby_many", "p3dfft_clean", "get_timers", "set_timers",
]

F64 = 0
F32 = 1
LAYOUT_XYZ = 0
LAYOUT_STRIDE1 = 1
SPEC_K2 = 1
SPEC_HERMITIAN = 2
JOB_ROUNDTRIP = 0
JOB_FORWARD = 1
JOB_BACKWARD = 2
JOB_SPECTRUM = 3
FLAG_TIMERS = 1
RANGE_FIXED = 0
RANGE_AUTO = 1
E_RANGE = -6


class P3DFFTError(RuntimeError):
    pass


def _core():
    return _lib.load().core


def _check(rc: int):
    if rc != 0:
        raise P3DFFTError(f"p3g error {rc}: {_core().p3g_last_error().decode()}")


def _ptr(t) -> int:
    """Data pointer of a torch tensor (device) or numpy array (host)."""
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def _stream_ptr(stream) -> int | None:
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except ImportError:
            pass
        return None
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class Plan:
    """Device plan for an nx*ny*nz grid (optionally pruned to nxc*nyc*nzc).

    ``precision`` is F64 (binary64 data, double-float arithmetic) or F32.
    Arrays are CUDA tensors in the reference's layouts: real (nz, ny, nx),
    complex (nzc, nyc, nxc//2+1) complex128/complex64 (or float views).
    """

    def __init__(self, nx, ny, nz, nxc=None, nyc=None, nzc=None, precision=F64, layout=LAYOUT_XYZ, timers=False,
                 max_radix=0, max_lines=0):
        self._h = ctypes.c_void_p()
        self.nx, self.ny, self.nz = nx, ny, nz
        self.nxc = nxc or nx
        self.nyc = nyc or ny
        self.nzc = nzc or nz
        self.precision = precision
        self.layout = layout
        self.tuning = (int(max_radix), int(max_lines))
        _check(_core().p3g_plan_create_tuned(ctypes.byref(self._h), nx, ny, nz, self.nxc, self.nyc, self.nzc,
                                             precision, layout, FLAG_TIMERS if timers else 0, int(max_radix),
                                             int(max_lines)))

    def work_bytes(self, kind) -> int:
        """Device work buffer a batch job of this kind needs (p3g_job_work_bytes)."""
        n = _core().p3g_job_work_bytes(self._h, int(kind))
        if n < 0:
            _check(-1)
        return n

    @property
    def real_shape(self):
        return (self.nz, self.ny, self.nx)

    @property
    def complex_shape(self):
        if self.layout == LAYOUT_STRIDE1:
            return (self.nxc // 2 + 1, self.nyc, self.nzc)
        return (self.nzc, self.nyc, self.nxc // 2 + 1)

    def get_dims(self, conf: int):
        s, e, z = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
        _check(_core().p3g_get_dims(self._h, conf, s, e, z))
        return tuple(s), tuple(e), tuple(z)

    def _dtypes(self):
        import torch
        return (torch.float64, torch.complex128) if self.precision == F64 else (torch.float32, torch.complex64)

    def ftran_r2c(self, x, out=None, op="fft", nv=1, dim_in=0, dim_out=0, stream=None):
        if out is None:
            import torch
            shape = ((nv,) if nv > 1 else ()) + self.complex_shape
            out = torch.empty(shape, dtype=self._dtypes()[1], device=x.device)
        _check(_core().p3g_ftran_r2c(self._h, _ptr(x), _ptr(out), op.encode(), nv, dim_in, dim_out,
                                     _stream_ptr(stream)))
        return out

    def btran_c2r(self, c, out=None, op="tff", nv=1, dim_in=0, dim_out=0, stream=None):
        if out is None:
            import torch
            shape = ((nv,) if nv > 1 else ()) + self.real_shape
            out = torch.empty(shape, dtype=self._dtypes()[0], device=c.device)
        _check(_core().p3g_btran_c2r(self._h, _ptr(c), _ptr(out), op.encode(), nv, dim_in, dim_out,
                                     _stream_ptr(stream)))
        return out

    def ftran_r2c_1d(self, x, out=None, stream=None):
        """The X r2c alone (p3g_ftran_r2c_1d): complex (nz, ny, nx//2+1), every mode."""
        if out is None:
            import torch
            out = torch.empty((self.nz, self.ny, self.nx // 2 + 1), dtype=self._dtypes()[1], device=x.device)
        _check(_core().p3g_ftran_r2c_1d(self._h, _ptr(x), _ptr(out), _stream_ptr(stream)))
        return out

    def cheby(self, x, lz, out=None, nv=1, dim_in=0, dim_out=0, stream=None):
        if out is None:
            import torch
            shape = ((nv,) if nv > 1 else ()) + self.complex_shape
            out = torch.empty(shape, dtype=self._dtypes()[1], device=x.device)
        _check(_core().p3g_cheby(self._h, _ptr(x), _ptr(out), float(lz), nv, dim_in, dim_out, _stream_ptr(stream)))
        return out

    def ftran_r2c_to_host(self, x, out_host, op="fft", chunks=8, stream=None, copy_stream=None):
        """Forward transform into a host (pinned) complex tensor, the host
        copies overlapped with the Z pass in row blocks (p3g_ftran_r2c_to_host)."""
        import torch
        dev = x.device if x.is_cuda else torch.device("cuda", torch.cuda.current_device())
        stage = torch.empty(self.complex_shape, dtype=self._dtypes()[1], device=dev)
        cs = copy_stream or torch.cuda.Stream(device=dev)
        st = _stream_ptr(stream)
        _check(_core().p3g_ftran_r2c_to_host(self._h, _ptr(x), _ptr(out_host), _ptr(stage), op.encode(), chunks, st,
                                             _stream_ptr(cs)))
        torch.cuda.synchronize(dev)
        return out_host

    def btran_c2r_from_host(self, c_host, out, op="tff", chunks=8, stream=None, copy_stream=None):
        """Backward transform of a host (pinned) complex tensor, the host copies
        overlapped with the Z pass in row blocks (p3g_btran_c2r_from_host)."""
        import torch
        dev = out.device if out.is_cuda else torch.device("cuda", torch.cuda.current_device())
        stage = torch.empty(self.complex_shape, dtype=self._dtypes()[1], device=dev)
        cs = copy_stream or torch.cuda.Stream(device=dev)
        _check(_core().p3g_btran_c2r_from_host(self._h, _ptr(c_host), _ptr(stage), _ptr(out), op.encode(), chunks,
                                               _stream_ptr(stream), _stream_ptr(cs)))
        torch.cuda.synchronize(dev)
        return out

    def spectrum(self, b, kmax=0, scale=1.0, flags=None, nv=1, dim_in=0, out=None, stream=None):
        """Shell spectrum of the forward output b (see p3g_spectrum); returns a
        float64 CUDA tensor of kmax + 1 bins (nv rows when nv > 1).  flags
        defaults to SPEC_K2, the spectrum sample's k^2 |B|^2 weighting."""
        import math
        import torch
        if flags is None:
            flags = SPEC_K2
        if kmax <= 0:
            kmax = int(math.sqrt(float(self.nx) ** 2 + float(self.ny) ** 2 + float(self.nz) ** 2) * 0.5 + 0.5)
        if out is None:
            shape = ((nv,) if nv > 1 else ()) + (kmax + 1,)
            out = torch.empty(shape, dtype=torch.float64, device=b.device)
        _check(_core().p3g_spectrum(self._h, _ptr(b), _ptr(out), kmax, float(scale), int(flags), nv, dim_in,
                                    _stream_ptr(stream)))
        return out

    def set_options(self, pipe=True, tma=True):
        """Kernel selection (see p3g_plan_set_options)."""
        _check(_core().p3g_plan_set_options(self._h, int(pipe), int(tma)))

    def check(self):
        """Synchronise and raise if a kernel recorded a failure or an F64
        transform's input was outside the exponent window (p3g_plan_status)."""
        _check(_core().p3g_plan_status(self._h))

    def block_tiles(self, on=True):
        """Test hook: the pipelined passes' tile waits run out (p3g_plan_block_tiles)."""
        _check(_core().p3g_plan_block_tiles(self._h, int(on)))

    def set_range(self, mode=RANGE_FIXED, bias=0):
        """Exponent bias of the F64 path (p3g_plan_set_range): RANGE_FIXED
        with inputs scaled by 2^-bias, or RANGE_AUTO (picked per call on the
        device from the input's largest magnitude)."""
        _check(_core().p3g_plan_set_range(self._h, int(mode), int(bias)))

    def check_range(self):
        """(rc, bias, emax) of p3g_plan_check_range: rc is 0 or E_RANGE, bias
        the exponent bias that brings the inputs since the last check into the
        window, emax their largest binary64 exponent."""
        b, e = ctypes.c_int(), ctypes.c_int()
        rc = _core().p3g_plan_check_range(self._h, ctypes.byref(b), ctypes.byref(e))
        if rc not in (0, E_RANGE):
            _check(rc)
        return rc, b.value, e.value

    def timers(self):
        t = (ctypes.c_double * 12)()
        _check(_core().p3g_get_timers(self._h, t))
        return list(t)

    def reset_timers(self):
        _check(_core().p3g_set_timers(self._h))

    @property
    def device_bytes(self) -> int:
        return _core().p3g_plan_device_bytes(self._h)

    @property
    def launches(self) -> int:
        return _core().p3g_plan_launches(self._h)

    def close(self):
        if self._h:
            _core().p3g_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent transforms in one persistent launch (p3g_batch_*).

    ``jobs`` is a list of dicts with keys plan (a Plan of this batch's
    precision), kind (JOB_*), in, out (CUDA tensors) and optionally kmax,
    scale, flags (spectrum jobs) and work (a uint8 CUDA tensor of at least
    plan.work_bytes(kind) bytes; allocated here when absent).  The tensors
    are bound until the next set_jobs.
    """

    def __init__(self, precision=F64):
        self.precision = precision
        self._h = ctypes.c_void_p()
        _check(_core().p3g_batch_create(ctypes.byref(self._h), precision))
        self._keep = []

    def set_jobs(self, jobs, window=0):
        import torch
        arr = (_lib.Job * len(jobs))()
        keep = []
        for i, j in enumerate(jobs):
            plan = j["plan"]
            work = j.get("work")
            if work is None:
                work = torch.empty(plan.work_bytes(j["kind"]), dtype=torch.uint8, device=j["in"].device)
            keep += [plan, j["in"], j["out"], work]
            arr[i].plan = plan._h.value
            arr[i].kind = int(j["kind"])
            arr[i].kmax = int(j.get("kmax", 0))
            arr[i].flags = int(j.get("flags", SPEC_K2))
            arr[i].scale = float(j.get("scale", 1.0))
            arr[i].in_ = _ptr(j["in"])
            arr[i].out = _ptr(j["out"])
            arr[i].work = _ptr(work)
        _check(_core().p3g_batch_set_jobs(self._h, len(jobs), arr, int(window)))
        self._keep = keep
        return self

    def launch(self, stream=None):
        _check(_core().p3g_batch_launch(self._h, _stream_ptr(stream)))

    def capture(self):
        _check(_core().p3g_batch_capture(self._h))

    def replay(self, stream=None):
        _check(_core().p3g_batch_replay(self._h, _stream_ptr(stream)))

    def check(self, stream=None):
        _check(_core().p3g_batch_status(self._h, _stream_ptr(stream)))

    def block_pass(self, index):
        """Test hook: the waits on pass `index` run out (p3g_batch_block_pass)."""
        _check(_core().p3g_batch_block_pass(self._h, int(index)))

    def info(self):
        a = (ctypes.c_longlong * 5)()
        _check(_core().p3g_batch_info(self._h, a))
        return {"passes": a[0], "items": a[1], "ctas": a[2], "launches": a[3], "threads": a[4]}

    def close(self):
        if self._h:
            _core().p3g_batch_destroy(self._h)
            self._h = ctypes.c_void_p()
        self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------------------
# reference module interface through the drop-in library
# ----------------------------------------------------------------------------
_single = False


def _legacy():
    libs = _lib.load()
    return libs.legacy_single if _single else libs.legacy


def _ci(v) -> ctypes.c_int:
    return ctypes.c_int(int(v))


def _legacy_check():
    lib = _legacy()
    st = lib.p3dfft_gb_status()
    if st != 0:
        raise P3DFFTError(lib.p3dfft_gb_last_error().decode())


def p3dfft_setup(dims, nx, ny, nz, comm=0, nxc=None, nyc=None, nzc=None, overwrite=True, single=False,
                 stride1=False):
    """setup.F90:107: returns memsize (the padded in-place size).  stride1
    selects the (nzc, nyc, nxhpc) output layout of the reference's STRIDE1
    build."""
    global _single
    _single = bool(single)
    d = (ctypes.c_int * 2)(*dims)
    mem = (ctypes.c_int * 3)()
    _legacy().p3dfft_gb_set_layout(LAYOUT_STRIDE1 if stride1 else LAYOUT_XYZ)
    _legacy_check()
    _legacy().p3dfft_setup(d, ctypes.byref(_ci(nx)), ctypes.byref(_ci(ny)), ctypes.byref(_ci(nz)),
                           ctypes.byref(_ci(comm)), ctypes.byref(_ci(nxc or nx)), ctypes.byref(_ci(nyc or ny)),
                           ctypes.byref(_ci(nzc or nz)), ctypes.byref(_ci(1 if overwrite else 0)), mem)
    _legacy_check()
    return tuple(mem)


def p3dfft_get_dims(conf: int):
    """module.F90:225: (start, end, size), 1-based, Fortran dimension order."""
    s, e, z = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
    _legacy().p3dfft_get_dims(s, e, z, ctypes.byref(_ci(conf)))
    _legacy_check()
    return tuple(s), tuple(e), tuple(z)


def p3dfft_get_mpi_info():
    t, n, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _legacy().p3dfft_get_mpi_info(ctypes.byref(t), ctypes.byref(n), ctypes.byref(c))
    _legacy_check()
    return t.value, n.value, c.value


def _real_dtype():
    return np.float32 if _single else np.float64


def _check_host(a, complex_=False):
    if hasattr(a, "data_ptr"):
        return
    want = (np.complex64 if _single else np.complex128) if complex_ else _real_dtype()
    if a.dtype != want or not a.flags.c_contiguous:
        raise P3DFFTError(f"array must be C-contiguous {np.dtype(want).name}")


def p3dfft_ftran_r2c(XgYZ, XYZg, op="fft"):
    _check_host(XgYZ)
    _check_host(XYZg, True)
    _legacy().p3dfft_ftran_r2c(_ptr(XgYZ), _ptr(XYZg), op.encode())
    _legacy_check()
    return XYZg


def p3dfft_btran_c2r(XYZg, XgYZ, op="tff"):
    _check_host(XYZg, True)
    _check_host(XgYZ)
    _legacy().p3dfft_btran_c2r(_ptr(XYZg), _ptr(XgYZ), op.encode())
    _legacy_check()
    return XgYZ


def p3dfft_ftran_r2c_many(XgYZ, dim_in, XYZg, dim_out, nv, op="fft"):
    _legacy().p3dfft_ftran_r2c_many(_ptr(XgYZ), ctypes.byref(_ci(dim_in)), _ptr(XYZg), ctypes.byref(_ci(dim_out)),
                                    ctypes.byref(_ci(nv)), op.encode())
    _legacy_check()
    return XYZg


def p3dfft_btran_c2r_many(XYZg, dim_in, XgYZ, dim_out, nv, op="tff"):
    _legacy().p3dfft_btran_c2r_many(_ptr(XYZg), ctypes.byref(_ci(dim_in)), _ptr(XgYZ), ctypes.byref(_ci(dim_out)),
                                    ctypes.byref(_ci(nv)), op.encode())
    _legacy_check()
    return XgYZ


def p3dfft_ftran_r2c_1d(rXgYZ, cXgYZ):
    """ftran.F90:787-814: the X r2c alone, real (nz, ny, nx) -> complex (nz, ny, nx//2+1)."""
    _check_host(rXgYZ)
    _check_host(cXgYZ, True)
    _legacy().p3dfft_ftran_r2c_1d(_ptr(rXgYZ), _ptr(cXgYZ))
    _legacy_check()
    return cXgYZ


def _lz_arg(lz):
    return ctypes.byref(ctypes.c_float(lz) if _single else ctypes.c_double(lz))


def p3dfft_cheby(XgYZ, XYZg, Lz):
    _legacy().p3dfft_cheby(_ptr(XgYZ), _ptr(XYZg), _lz_arg(Lz))
    _legacy_check()
    return XYZg


def p3dfft_cheby_many(XgYZ, dim_in, XYZg, dim_out, nv, Lz):
    _legacy().p3dfft_cheby_many(_ptr(XgYZ), ctypes.byref(_ci(dim_in)), _ptr(XYZg), ctypes.byref(_ci(dim_out)),
                                ctypes.byref(_ci(nv)), _lz_arg(Lz))
    _legacy_check()
    return XYZg


def p3dfft_clean():
    _legacy().p3dfft_clean()


def get_timers():
    t = (ctypes.c_double * 12)()
    _legacy().get_timers(t)
    return list(t)


def set_timers():
    _legacy().set_timers()
