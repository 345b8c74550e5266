"""Loads the in-tree shared libraries and declares their C signatures."""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_double_p = ctypes.POINTER(ctypes.c_double)

class Job(ctypes.Structure):
    """p3g_job (include/p3dfft_gb300.h)."""
    _fields_ = [("plan", ctypes.c_void_p), ("kind", ctypes.c_int), ("kmax", ctypes.c_int),
                ("flags", ctypes.c_int), ("reserved", ctypes.c_int), ("scale", ctypes.c_double),
                ("in_", ctypes.c_void_p), ("out", ctypes.c_void_p), ("work", ctypes.c_void_p)]


# explicit device API (include/p3dfft_gb300.h)
CORE_SIGNATURES = {
    "p3g_plan_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int]),
    "p3g_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "p3g_get_dims": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _c_int_p, _c_int_p, _c_int_p]),
    "p3g_ftran_r2c": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                     ctypes.c_int, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_void_p]),
    "p3g_btran_c2r": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                     ctypes.c_int, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_void_p]),
    "p3g_cheby": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                 ctypes.c_longlong, ctypes.c_longlong, ctypes.c_void_p]),
    "p3g_ftran_r2c_1d": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "p3g_get_timers": (ctypes.c_int, [ctypes.c_void_p, _c_double_p]),
    "p3g_set_timers": (ctypes.c_int, [ctypes.c_void_p]),
    "p3g_plan_device_bytes": (ctypes.c_longlong, [ctypes.c_void_p]),
    "p3g_plan_launches": (ctypes.c_longlong, [ctypes.c_void_p]),
    "p3g_ftran_r2c_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                             ctypes.c_void_p]),
    "p3g_plan_status": (ctypes.c_int, [ctypes.c_void_p]),
    "p3g_plan_set_range": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "p3g_plan_block_tiles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "p3g_plan_check_range": (ctypes.c_int, [ctypes.c_void_p, _c_int_p, _c_int_p]),
    "p3g_plan_create_tuned": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "p3g_job_work_bytes": (ctypes.c_longlong, [ctypes.c_void_p, ctypes.c_int]),
    "p3g_ftran_r2c_to_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "p3g_btran_c2r_from_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "p3g_batch_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]),
    "p3g_batch_set_jobs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Job), ctypes.c_int]),
    "p3g_batch_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "p3g_batch_capture": (ctypes.c_int, [ctypes.c_void_p]),
    "p3g_batch_replay": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "p3g_batch_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "p3g_batch_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "p3g_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "p3g_batch_block_pass": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "p3g_spectrum": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p]),
    "p3g_plan_set_options": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "p3g_last_error": (ctypes.c_char_p, []),
    "p3g_version": (ctypes.c_int, []),
}

# drop-in reference API (include/p3dfft.h); every argument by pointer
LEGACY_SIGNATURES = {
    "p3dfft_setup": (None, [_c_int_p, _c_int_p, _c_int_p, _c_int_p, _c_int_p, _c_int_p, _c_int_p, _c_int_p,
                            _c_int_p, _c_int_p]),
    "p3dfft_get_dims": (None, [_c_int_p, _c_int_p, _c_int_p, _c_int_p]),
    "p3dfft_get_mpi_info": (None, [_c_int_p, _c_int_p, _c_int_p]),
    "p3dfft_ftran_r2c": (None, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p]),
    "p3dfft_btran_c2r": (None, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p]),
    "p3dfft_ftran_r2c_many": (None, [ctypes.c_void_p, _c_int_p, ctypes.c_void_p, _c_int_p, _c_int_p,
                                     ctypes.c_char_p]),
    "p3dfft_btran_c2r_many": (None, [ctypes.c_void_p, _c_int_p, ctypes.c_void_p, _c_int_p, _c_int_p,
                                     ctypes.c_char_p]),
    "p3dfft_ftran_r2c_1d": (None, [ctypes.c_void_p, ctypes.c_void_p]),
    "p3dfft_cheby": (None, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "p3dfft_cheby_many": (None, [ctypes.c_void_p, _c_int_p, ctypes.c_void_p, _c_int_p, _c_int_p,
                                 ctypes.c_void_p]),
    "p3dfft_clean": (None, []),
    "get_timers": (None, [_c_double_p]),
    "set_timers": (None, []),
    "p3dfft_gb_status": (ctypes.c_int, []),
    "p3dfft_gb_last_error": (ctypes.c_char_p, []),
    "p3dfft_gb_set_abort": (None, [ctypes.c_int]),
    "p3dfft_gb_set_layout": (None, [ctypes.c_int]),
}


class Libraries:
    def __init__(self, core, legacy, legacy_single):
        self.core = core
        self.legacy = legacy
        self.legacy_single = legacy_single


_LIBS = None


def _declare(lib, sigs):
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def load(build_if_missing: bool = True) -> Libraries:
    """Load (building first if needed) the three libraries.  Raises if the
    CUDA toolchain or the libraries are missing: there is no CPU fallback."""
    global _LIBS
    if _LIBS is not None:
        return _LIBS
    paths = {k: _build.lib_path(k) for k in _build.LIBS}
    if not all(os.path.exists(p) for p in paths.values()):
        if not build_if_missing:
            raise RuntimeError("p3dfft_gb300 libraries are not built; run __graft_entry__.build()")
        paths = _build.build()
    core = ctypes.CDLL(paths["core"], mode=ctypes.RTLD_GLOBAL)
    _declare(core, CORE_SIGNATURES)
    legacy = ctypes.CDLL(paths["legacy"])
    _declare(legacy, LEGACY_SIGNATURES)
    single = ctypes.CDLL(paths["legacy_single"])
    _declare(single, LEGACY_SIGNATURES)
    legacy.p3dfft_gb_set_abort(0)
    single.p3dfft_gb_set_abort(0)
    _LIBS = Libraries(core, legacy, single)
    return _LIBS
