"""CPU oracle for the P3DFFT 3D transform path (TEST INFRASTRUCTURE ONLY).

This module is the checker, not the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it.  The shipped library (``p3dfft_gb300``) never calls into it and has no CPU
fallback.

It restates, step by step and in FP64 numpy/scipy (pocketfft), what the
reference P3DFFT 2.7 library computes on a single rank with a 1x1 processor
grid in its default build (FFTW backend, non-STRIDE1 output layout, optional
STRIDE1 layout as a flag):

* ``p3dfft_ftran_r2c``   build/ftran.F90:489-780
* ``p3dfft_btran_c2r``   build/btran.F90:396-679
* ``p3dfft_cheby``       build/ftran.F90:383-464
* ``p3dfft_*_many``      build/ftran.F90:104-317, build/btran.F90:104-304
  (restated as nv independent single-variable transforms; see ``ftran_many``)
* ``p3dfft_get_dims``    build/module.F90:225-273
* ``MapDataToProc``      build/setup.F90:608-635
* pruning copies         build/module.F90:502-556 (seg_zero_*), :649-706 (seg_copy_*)
* shell spectrum         sample/FORTRAN/driver_spec.F90:263-341

FFTW conventions restated (the library the reference calls, not vendored in
the reference tree and not version pinned by it, configure.ac:330-353):
r2c/c2r and c2c are unnormalised, forward sign exp(-i), backward exp(+i); c2r
ignores the imaginary parts of the DC and Nyquist bins; REDFT00 (DCT-I) and
RODFT00 (DST-I) are unnormalised.  numpy/scipy pocketfft follows the same
conventions (checked in tests/test_oracle.py).

Array convention: numpy C-order arrays with the Fortran dimensions reversed,
so the reference's real input ``XgYZ(nx,ny,nz)`` is an ``(nz, ny, nx)`` array
and its complex output ``XYZg(nxhpc,nyc,nzc)`` is ``(nzc, nyc, nxhpc)`` (or
``(nxhpc, nyc, nzc)`` for the STRIDE1 layout ``XYZg(nzc,nyc,nxhpc)``).

Parity status: pinned against every analytic known-answer check the reference
sample programs contain (tests/test_oracle.py); FFTW-bitwise parity is not
pinned because the reference cannot be built in this environment (no Fortran
compiler, MPI or FFTW).
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sfft

# Worker threads for scipy.fft (the CPU-baseline leg sets this to the core count).
WORKERS = 1

VALID_OPS = ("t", "f", "c", "s", "n", "0")


class OracleError(ValueError):
    """Raised where the reference prints an error and calls MPI_Abort."""


# --------------------------------------------------------------------------
# integer layout logic
# --------------------------------------------------------------------------
def map_data_to_proc(data: int, proc: int):
    """Block mapping of ``data`` points onto ``proc`` ranks (setup.F90:608-635).

    Returns 1-based (start, end, size) lists of length ``proc``: the first
    ``proc - data % proc`` ranks get ``data // proc`` points, the rest one more.
    """
    size = data // proc
    nu = data - size * proc
    nl = proc - nu
    st = [0] * proc
    en = [0] * proc
    sz = [0] * proc
    st[0] = 1
    sz[0] = size
    en[0] = size
    for i in range(1, nl):
        st[i] = st[i - 1] + size
        sz[i] = size
        en[i] = en[i - 1] + size
    size += 1
    for i in range(max(nl, 1), proc):
        st[i] = en[i - 1] + 1
        sz[i] = size
        en[i] = en[i - 1] + size
    en[proc - 1] = data
    sz[proc - 1] = data - st[proc - 1] + 1
    return st, en, sz


class OraclePlan:
    """State set by ``p3dfft_setup`` (setup.F90:107-605) for one rank.

    ``dims`` is the processor grid (iproc, jproc); ``rank`` selects the rank
    whose local bounds ``get_dims`` reports.  Transforms are only restated for
    the 1x1 grid, which is the whole global array.
    """

    def __init__(self, nx, ny, nz, nxc=None, nyc=None, nzc=None, overwrite=True,
                 dims=(1, 1), rank=0, stride1=False):
        if nx <= 0 or ny <= 0 or nz <= 0:
            raise OracleError(f"Invalid dimensions : {nx} {ny} {nz}")  # setup.F90:125-128
        iproc, jproc = dims
        nproc = iproc * jproc
        if iproc <= 0 or jproc <= 0:
            raise OracleError(f"Invalid processor geometry: {dims}")  # setup.F90:181-184
        self.nx, self.ny, self.nz = nx, ny, nz
        self.nxc = nx if nxc is None else nxc
        self.nyc = ny if nyc is None else nyc
        self.nzc = nz if nzc is None else nzc
        self.overwrite = bool(overwrite)
        self.stride1 = stride1
        self.iproc, self.jproc = iproc, jproc
        # derived sizes, setup.F90:160-170
        self.nxh = nx // 2
        self.nxhp = self.nxh + 1
        self.nxhc = self.nxc // 2
        self.nxhpc = self.nxhc + 1
        self.nyh = ny // 2
        self.nzh = nz // 2
        self.nyhc = self.nyc // 2
        self.nzhc = self.nzc // 2
        self.nycph = (self.nyc + 1) // 2
        self.nzcph = (self.nzc + 1) // 2
        # rank coordinates without DIMS_C: MPI_Cart_create on (jproc, iproc),
        # ipid = cartid(2), jpid = cartid(1) (setup.F90:194-231)
        self.ipid = rank % iproc
        self.jpid = rank // iproc
        self.nproc = nproc
        self.iist, self.iien, self.iisz = map_data_to_proc(self.nxhpc, iproc)
        self.jist, self.jien, self.jisz = map_data_to_proc(ny, iproc)
        self.jjst, self.jjen, self.jjsz = map_data_to_proc(self.nyc, jproc)
        self.kjst, self.kjen, self.kjsz = map_data_to_proc(nz, jproc)
        ip, jp = self.ipid, self.jpid
        self.iistart, self.iiend, self.iisize = self.iist[ip], self.iien[ip], self.iisz[ip]
        self.jjstart, self.jjend, self.jjsize = self.jjst[jp], self.jjen[jp], self.jjsz[jp]
        self.jistart, self.jiend, self.jisize = self.jist[ip], self.jien[ip], self.jisz[ip]
        self.kjstart, self.kjend, self.kjsize = self.kjst[jp], self.kjen[jp], self.kjsz[jp]
        # memsize / padded bounds, setup.F90:579-603
        pad1 = 2 * max(nz * self.jjsize * self.iisize, ny * self.kjsize * self.iisize) \
            - nx * self.jisize * self.kjsize
        pad1 = max(pad1, 0)
        denom = nx * self.jisize
        padi = pad1 // denom + (1 if pad1 % denom else 0) if denom else 0
        self.maxisize = nx
        self.maxjsize = self.jisize
        self.maxksize = self.kjsize + padi
        self.memsize = (self.maxisize, self.maxjsize, self.maxksize)

    # module.F90:225-273
    def get_dims(self, conf: int):
        if conf == 1:
            return ((1, self.jistart, self.kjstart), (self.nx, self.jiend, self.kjend),
                    (self.nx, self.jisize, self.kjsize))
        if conf == 2:
            if self.stride1:
                return ((1, self.jjstart, self.iistart), (self.nzc, self.jjend, self.iiend),
                        (self.nzc, self.jjsize, self.iisize))
            return ((self.iistart, self.jjstart, 1), (self.iiend, self.jjend, self.nzc),
                    (self.iisize, self.jjsize, self.nzc))
        if conf == 3:
            return ((0, 0, 0), self.memsize, self.memsize)
        raise OracleError(f"unknown conf {conf}")

    # ------------------------------------------------------------------
    # transforms (1x1 grid only)
    # ------------------------------------------------------------------
    def _check_1x1(self):
        if self.iproc != 1 or self.jproc != 1:
            raise OracleError("transforms are restated for the 1x1 processor grid only")

    def _zop(self, a: np.ndarray, ch: str, forward: bool) -> np.ndarray:
        """Z transform selected by one op letter, along axis 0 (ftran.F90:620-643)."""
        if ch in ("t", "f"):
            if forward:
                return sfft.fft(a, axis=0, workers=WORKERS, overwrite_x=True)
            return sfft.ifft(a, axis=0, norm="forward", workers=WORKERS, overwrite_x=True)
        if ch == "c":  # REDFT00 on re and im parts (fft_exec.F90:646-701)
            if a.shape[0] < 2:
                raise OracleError("DCT-I needs nz >= 2")
            return sfft.dct(a, type=1, axis=0, workers=WORKERS)
        if ch == "s":  # RODFT00 (fft_exec.F90:866-921)
            return sfft.dst(a, type=1, axis=0, workers=WORKERS)
        if ch in ("n", "0"):
            return a
        raise OracleError(f"Unknown transform type: {ch}")

    def ftran_r2c(self, x: np.ndarray, op: str = "fft") -> np.ndarray:
        """Forward r2c, ftran.F90:489-780 at iproc = jproc = 1."""
        self._check_1x1()
        op = _normalise_op(op)
        x = np.asarray(x, dtype=np.float64)
        if x.shape != (self.nz, self.ny, self.nx):
            raise OracleError(f"input shape {x.shape} != {(self.nz, self.ny, self.nx)}")
        # X r2c into buf2 (ftran.F90:525-534)
        buf2 = sfft.rfft(x, axis=2, workers=WORKERS)
        # seg_copy_x keeps x modes 1..nxhpc (ftran.F90:554); a copy only when pruned
        buf = np.ascontiguousarray(buf2[:, :, : self.nxhpc])
        del buf2
        # Y c2c per z-plane (ftran.F90:576-584)
        buf = sfft.fft(buf, axis=1, workers=WORKERS, overwrite_x=True)
        # seg_copy_y: y = 1..nycph from y, y = nycph+1..nyc from y+dny (ftran.F90:736-738)
        dny = self.ny - self.nyc
        if dny == 0:
            b1 = buf  # the identity copy
        else:
            b1 = np.empty((self.nz, self.nyc, self.nxhpc), dtype=np.complex128)
            b1[:, : self.nycph] = buf[:, : self.nycph]
            b1[:, self.nycph:] = buf[:, self.nycph + dny: self.nyc + dny]
        del buf
        # Z op over the full nz (ftran.F90:740-763)
        b1 = self._zop(b1, op[2], forward=True)
        # seg_copy_z: z = 1..nzcph from z, z = nzcph+1..nzc from z+dnz (ftran.F90:705-706)
        dnz = self.nz - self.nzc
        if dnz == 0:
            out = b1
        else:
            out = np.empty((self.nzc, self.nyc, self.nxhpc), dtype=np.complex128)
            out[: self.nzcph] = b1[: self.nzcph]
            out[self.nzcph:] = b1[self.nzcph + dnz: self.nzc + dnz]
        if self.stride1:
            out = np.ascontiguousarray(out.transpose(2, 1, 0))
        return out

    def btran_c2r(self, c: np.ndarray, op: str = "tff") -> np.ndarray:
        """Backward c2r, btran.F90:396-679 at iproc = jproc = 1.

        The overwrite (OW) branch with nz == nzc (btran.F90:525-550) differs
        from the general branch only in where the Z op runs; both give the same
        result when nyc == ny.  With nyc < ny that branch copies an
        (nxhpc, nyc, nz) block into a buffer read as (nxhpc, ny, nz) and so
        reads stale workspace; this restatement uses the general branch's
        zero-filled y copy for every case.
        """
        self._check_1x1()
        op = _normalise_op(op)
        c = np.asarray(c)
        if self.stride1:
            if c.shape != (self.nxhpc, self.nyc, self.nzc):
                raise OracleError(f"input shape {c.shape}")
            c = c.transpose(2, 1, 0)
        if c.shape != (self.nzc, self.nyc, self.nxhpc):
            raise OracleError(f"input shape {c.shape} != {(self.nzc, self.nyc, self.nxhpc)}")
        nz, ny, nzc, nyc = self.nz, self.ny, self.nzc, self.nyc
        dnz = nz - nzc
        # seg_copy_z low, seg_copy_z high, seg_zero_z (btran.F90:553-555); the
        # input is never modified (every path below works on a copy)
        buf1 = np.empty((nz, nyc, self.nxhpc), dtype=np.complex128)
        buf1[: self.nzcph] = c[: self.nzcph]
        buf1[nz - self.nzcph:] = c[nz - self.nzcph - dnz: nz - dnz]
        buf1[self.nzcph: nz - self.nzcph] = 0
        buf1 = self._zop(buf1, op[0], forward=False)
        # seg_copy_y low/high + seg_zero_y (btran.F90:585-588)
        dny = ny - nyc
        if dny == 0:
            buf = buf1
        else:
            buf = np.empty((nz, ny, self.nxhpc), dtype=np.complex128)
            buf[:, : self.nycph] = buf1[:, : self.nycph]
            buf[:, ny - self.nycph:] = buf1[:, ny - self.nycph - dny: ny - dny]
            buf[:, self.nycph: ny - self.nycph] = 0
        del buf1
        # Y c2c backward (btran.F90:615-624)
        buf = sfft.ifft(buf, axis=1, norm="forward", workers=WORKERS, overwrite_x=True)
        # seg_copy_x + seg_zero_x (btran.F90:662-663)
        if self.nxhpc == self.nxhp:
            b1 = buf
        else:
            b1 = np.zeros((nz, ny, self.nxhp), dtype=np.complex128)
            b1[:, :, : self.nxhpc] = buf
        del buf
        # X c2r (btran.F90:665-670), unnormalised
        return sfft.irfft(b1, n=self.nx, axis=2, norm="forward", workers=WORKERS, overwrite_x=True)

    def cheby(self, x: np.ndarray, lz: float) -> np.ndarray:
        """p3dfft_cheby, ftran.F90:383-464: 'ffc' transform, 1/(nx*ny*(nzc-1))
        scaling, then the Chebyshev-derivative recurrence along z."""
        out = self.ftran_r2c(x, "ffc")
        if self.stride1:
            out = out.transpose(2, 1, 0)
        out = out * (1.0 / (float(self.nx * self.ny) * float(self.nzc - 1)))
        lfac = 4.0 / float(lz)
        n = self.nzc
        old = out[n - 2].copy()
        out[n - 2] = lfac * float(n - 1) * out[n - 1] * 0.5
        out[n - 1] = 0
        for k in range(n - 3, -1, -1):  # Fortran k = nzc-2 .. 1
            new = out[k].copy()
            out[k] = lfac * float(k + 1) * old + out[k + 2]
            old = new
        out[0] = out[0] * 0.5
        if self.stride1:
            out = np.ascontiguousarray(out.transpose(2, 1, 0))
        return out

    # _many variants as nv independent transforms
    def ftran_many(self, xs, op="fft"):
        """p3dfft_ftran_r2c_many (ftran.F90:104-317) restated as independent
        single-variable transforms.  The reference's multi-variable code keeps
        nyhc/nzhc low modes where the single-variable code keeps nycph/nzcph
        (ftran.F90:260-261,292-293); the two agree for even pruned sizes."""
        return np.stack([self.ftran_r2c(x, op) for x in xs])

    def btran_many(self, cs, op="tff"):
        """p3dfft_btran_c2r_many (btran.F90:104-304) restated as independent
        single-variable transforms (the reference's 1x1 pruned branch reads
        buf1 after transforming buf, btran.F90:222-226)."""
        return np.stack([self.btran_c2r(c, op) for c in cs])


def _normalise_op(op) -> str:
    if isinstance(op, bytes):
        op = op.decode("ascii")
    op = str(op)
    if len(op) < 3:
        raise OracleError(f"op must have 3 letters, got {op!r}")
    return op[:3]


# --------------------------------------------------------------------------
# caller-side pieces used by the sample programs
# --------------------------------------------------------------------------
def shell_spectrum(b: np.ndarray, nx: int, ny: int, nz: int, stride1: bool = False, k2_weight: bool = True,
                   hermitian: bool = False, kmax: int = 0) -> np.ndarray:
    """compute_spectrum, driver_spec.F90:263-341, single rank.

    ``b`` is the (normalised) forward output in the ip=2 layout.  Returns
    E(0..kmax) with kmax = int(sqrt(nx^2+ny^2+nz^2)*0.5+0.5) by default
    (driver_spec.F90:198), E(ik) = sum k^2 |B|^2, ik = int(sqrt(k^2)+0.5); the
    r2c half is not doubled.  k2_weight=False gives unit weights and
    hermitian=True doubles the modes 0 < kx, 2 kx != nx (the conjugate half of
    a real field), the power spectrum of the serving form; modes with
    ik > kmax are not counted.
    """
    if kmax <= 0:
        kmax = int(np.sqrt(float(nx) * nx + ny * ny + nz * nz) * 0.5 + 0.5)
    if stride1:
        b = b.transpose(2, 1, 0)
    nzc, nyc, nxhpc = b.shape
    kz = np.arange(1, nzc + 1)
    kz = np.where(kz > nz // 2, nz - kz + 1, kz - 1)
    ky = np.arange(1, nyc + 1)
    ky = np.where(ky > ny // 2, ny - ky + 1, ky - 1)
    kx = np.arange(nxhpc)
    k2 = (kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2).astype(np.float64)
    ik = (np.sqrt(k2) + 0.5).astype(np.int64)
    w = b.real.astype(np.float64) ** 2 + b.imag.astype(np.float64) ** 2
    if k2_weight:
        w = k2 * w
    if hermitian:
        kxb = np.broadcast_to(kx[None, None, :], w.shape)
        w = np.where((kxb > 0) & (2 * kxb != nx), 2.0 * w, w)
    keep = ik <= kmax
    return np.bincount(ik[keep].ravel(), weights=w[keep].ravel(), minlength=kmax + 1)[: kmax + 1]


def normalised_linf(a: np.ndarray, ref: np.ndarray) -> float:
    """max|a - ref| / max|ref| (0 when both are zero)."""
    den = float(np.max(np.abs(ref))) if ref.size else 0.0
    num = float(np.max(np.abs(np.asarray(a) - ref))) if ref.size else 0.0
    return num / den if den > 0 else num


def relative_l2(a: np.ndarray, ref: np.ndarray) -> float:
    den = float(np.linalg.norm(ref.ravel()))
    num = float(np.linalg.norm((np.asarray(a) - ref).ravel()))
    return num / den if den > 0 else num


def roundtrip_tolerance(nglob: int, single: bool = False) -> float:
    """The samples' pass rule: max-abs error <= prec * Nglob * 0.25 with
    prec = 1e-14 (FP64) or 1e-5 (FP32) (driver_rand.F90:264-276)."""
    return (1e-5 if single else 1e-14) * nglob * 0.25
