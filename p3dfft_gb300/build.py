"""Builds the in-tree shared libraries for sm_103a (GB300).

Outputs, under ``p3dfft_gb300/_lib/``:

* ``libp3dfft_gb300.so``   kernels + plan + explicit device C-ABI (include/p3dfft_gb300.h)
* ``libp3dfft.so``         drop-in reference ABI, binary64 arrays (include/p3dfft.h)
* ``libp3dfft_single.so``  drop-in reference ABI, binary32 arrays (-DSINGLE_PREC)

Translation units compile in parallel with nvcc; a stamp of the source
hashes and flags skips the build when nothing changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
CORE_SOURCES = ["p3g_kernels_f64.cu", "p3g_kernels_f32.cu", "p3g_plan.cu", "p3g_noalloc.cu", "p3g_spectrum.cu",
                "p3g_batch.cu", "p3g_batch_f64_128.cu", "p3g_batch_f64_256.cu", "p3g_batch_f32_128.cu",
                "p3g_batch_f32_256.cu"]
LEGACY_SOURCE = "p3g_legacy.cpp"
LIBS = {
    "core": "libp3dfft_gb300.so",
    "legacy": "libp3dfft.so",
    "legacy_single": "libp3dfft_single.so",
}


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build p3dfft_gb300")


def _stamp() -> str:
    h = hashlib.sha256()
    h.update(" ".join(NVCC_FLAGS).encode())
    for d in (CSRC, os.path.join(ROOT, "include")):
        for name in sorted(os.listdir(d)):
            path = os.path.join(d, name)
            if os.path.isfile(path):
                h.update(name.encode())
                with open(path, "rb") as f:
                    h.update(f.read())
    with open(os.path.abspath(__file__), "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def lib_path(kind: str) -> str:
    return os.path.join(OUT, LIBS[kind])


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build command failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res


def build(force: bool = False, verbose: bool = False) -> dict:
    """Compile everything (if sources changed) and return the library paths."""
    os.makedirs(OBJ, exist_ok=True)
    stamp_file = os.path.join(OUT, "build.stamp")
    stamp = _stamp()
    paths = {k: lib_path(k) for k in LIBS}
    if (not force and os.path.exists(stamp_file) and all(os.path.exists(p) for p in paths.values())
            and open(stamp_file).read().strip() == stamp):
        return paths
    nvcc = nvcc_path()
    jobs = []
    for src in CORE_SOURCES:
        obj = os.path.join(OBJ, src + ".o")
        jobs.append([nvcc, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj])
    leg_d = os.path.join(OBJ, "legacy_f64.o")
    leg_s = os.path.join(OBJ, "legacy_f32.o")
    jobs.append([nvcc, *NVCC_FLAGS, "-c", os.path.join(CSRC, LEGACY_SOURCE), "-o", leg_d])
    jobs.append([nvcc, *NVCC_FLAGS, "-DSINGLE_PREC", "-c", os.path.join(CSRC, LEGACY_SOURCE), "-o", leg_s])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for res in ex.map(_run, jobs):
            if verbose and (res.stdout or res.stderr):
                print(res.stdout + res.stderr)
    core_objs = [os.path.join(OBJ, s + ".o") for s in CORE_SOURCES]
    _run([nvcc, *ARCH, "-shared", "-o", paths["core"], *core_objs, "-lcudart"])
    rpath = ["-Xlinker", "-rpath,$ORIGIN"]
    _run([nvcc, *ARCH, "-shared", "-o", paths["legacy"], leg_d, "-L" + OUT, "-lp3dfft_gb300", "-lcudart", *rpath])
    _run([nvcc, *ARCH, "-shared", "-o", paths["legacy_single"], leg_s, "-L" + OUT, "-lp3dfft_gb300", "-lcudart",
          *rpath])
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return paths


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
