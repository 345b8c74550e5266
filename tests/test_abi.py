"""C-ABI checks that need no GPU: the libraries load and export every
function the public headers declare."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"FORT_MOD_NAME\((\w+)\)\s*\(", text))
    for m in re.finditer(r"^\s*(?:extern\s+)?(?:const\s+)?[\w\*]+\s+\**(\w+)\s*\(", text, flags=re.M):
        if m.group(1) not in ("if", "return", "FORT_MOD_NAME"):
            names.add(m.group(1))
    return {n for n in names if not n.startswith("C")}  # Cp3dfft_* / Cget_timers are header-inline


def test_libraries_export_declared_symbols(lib):
    core_syms = _declared("p3dfft_gb300.h")
    assert "p3g_ftran_r2c" in core_syms and "p3g_plan_create" in core_syms
    for name in core_syms:
        assert hasattr(lib.core, name), name
    legacy_syms = _declared("p3dfft.h")
    for name in ("p3dfft_setup", "p3dfft_get_dims", "p3dfft_ftran_r2c", "p3dfft_btran_c2r", "p3dfft_clean",
                 "p3dfft_ftran_r2c_many", "p3dfft_btran_c2r_many", "p3dfft_cheby", "p3dfft_cheby_many",
                 "get_timers", "set_timers", "p3dfft_ftran_r2c_1d"):
        assert name in legacy_syms, name
    for name in legacy_syms:
        assert hasattr(lib.legacy, name), name
        assert hasattr(lib.legacy_single, name), name


def test_version_and_error_without_gpu(lib):
    assert lib.core.p3g_version() >= 100
    # no plan: get_dims reports a state error without touching the GPU
    s = (ctypes.c_int * 3)()
    assert lib.core.p3g_get_dims(None, 1, s, s, s) == -5
    assert b"setup" in lib.core.p3g_last_error()


def test_plan_rejects_bad_sizes_without_gpu(lib):
    h = ctypes.c_void_p()
    assert lib.core.p3g_plan_create(ctypes.byref(h), 0, 4, 4, 0, 0, 0, 0, 0, 0) == -1
    assert b"Invalid dimensions" in lib.core.p3g_last_error()
    assert lib.core.p3g_plan_create(ctypes.byref(h), 8, 8, 8, 10, 8, 8, 0, 0, 0) == -1
    assert lib.core.p3g_plan_create(ctypes.byref(h), 8, 8, 8, 8, 8, 8, 7, 0, 0) == -1
    # a plane of 2^31 or more elements (131072/2+1 modes x 32768 rows) is refused before any
    # device work: single per-element strides are 32-bit kernel parameters
    assert lib.core.p3g_plan_create(ctypes.byref(h), 131072, 32768, 2, 0, 0, 0, 0, 0, 0) == -4
    assert b"2^31" in lib.core.p3g_last_error()


def test_legacy_use_before_setup_prints_and_returns(lib):
    s = (ctypes.c_int * 3)()
    conf = ctypes.c_int(1)
    lib.legacy.p3dfft_get_dims(s, s, s, ctypes.byref(conf))
    assert lib.legacy.p3dfft_gb_status() == -5
    assert b"call setup before other routines" in lib.legacy.p3dfft_gb_last_error()


def test_legacy_rejects_multi_rank_geometry(lib):
    dims = (ctypes.c_int * 2)(2, 2)
    v = [ctypes.c_int(x) for x in (16, 16, 16, 0, 16, 16, 16, 1)]
    mem = (ctypes.c_int * 3)()
    lib.legacy.p3dfft_setup(dims, *[ctypes.byref(x) for x in v], mem)
    assert lib.legacy.p3dfft_gb_status() == -1
    assert b"Invalid processor geometry" in lib.legacy.p3dfft_gb_last_error()


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "p3dfft.h"\n#include "p3dfft_gb300.h"\n'
                   'int main(void){int d[2]={1,1},m[3];Cp3dfft_setup(d,8,8,8,0,8,8,8,1,m);return 0;}\n')
    res = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-c", "-I", os.path.join(ROOT, "include"),
                          str(src), "-o", str(tmp_path / "t.o")], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


def test_fortran_module_binds_exported_symbols(lib):
    # include/p3dfft.F90 (not compiled here: no Fortran compiler) binds every
    # routine to a C symbol of the drop-in libraries
    text = open(os.path.join(ROOT, "include", "p3dfft.F90")).read()
    names = re.findall(r"bind\(C,\s*name='(\w+)'\)", text)
    assert {"p3dfft_setup", "p3dfft_ftran_r2c", "p3dfft_btran_c2r", "p3dfft_get_dims", "p3dfft_clean",
            "p3dfft_cheby", "get_timers", "set_timers"} <= set(names)
    for name in names:
        assert hasattr(lib.legacy, name), name
        assert hasattr(lib.legacy_single, name), name
    # the reference module's public names are all there
    for name in ("p3dfft_type", "r8", "i8", "timers", "p3dfft_setup", "p3dfft_get_dims", "p3dfft_ftran_r2c",
                 "p3dfft_btran_c2r", "p3dfft_ftran_r2c_many", "p3dfft_btran_c2r_many", "p3dfft_cheby",
                 "p3dfft_cheby_many", "p3dfft_clean", "get_timers", "set_timers", "p3dfft_get_mpi_info",
                 "p3dfft_ftran_r2c_1d"):
        assert re.search(r"public\s*::[^\n]*\b%s\b" % name, text), name
