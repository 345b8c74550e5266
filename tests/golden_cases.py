"""Checks of a transform implementation against the committed closed-form
fixtures in tests/golden/known_answers.npz (made by make_golden.py).  `impl`
is a factory (nx, ny, nz) -> object with ftran(a, op), btran(c, op) and
cheby(a, lz) in the reference's array layouts (numpy in, numpy out)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers.npz")


def load():
    return np.load(GOLDEN)


def check_all(impl, tol):
    """tol: normalised L-inf bound for the forward spectra and the inverse."""
    g = load()
    for tag in ("14x26x38", "16x12x10"):
        nx, ny, nz = map(int, tag.split("x"))
        t = impl(nx, ny, nz)
        b = t.ftran(g[f"sine_{tag}_in"], "fft")
        want = g[f"sine_{tag}_out"]
        assert np.abs(b - want).max() <= tol * np.abs(want).max(), tag
    t = impl(16, 16, 16)
    r = t.btran(g["spikes_16x16x16_in"], "tff")
    want = g["spikes_16x16x16_out"]
    assert np.abs(r - want).max() <= tol * np.abs(want).max()
    t = impl(12, 8, 17)
    b = t.ftran(g["dct_12x8x17_m5_in"], "ffc")
    want = g["dct_12x8x17_m5_out"]
    assert np.abs(b - want).max() <= tol * np.abs(want).max()
    t = impl(12, 8, 15)
    b = t.ftran(g["dst_12x8x15_m4_in"], "ffs")
    want = g["dst_12x8x15_m4_out"]
    assert np.abs(b - want).max() <= tol * np.abs(want).max()
    # the Chebyshev sample's procedure and pass rule (driver_cheby.F90:218-284)
    nx, ny, nz = 8, 8, 33
    t = impl(nx, ny, nz)
    c = t.cheby(g["cheby_8x8x33_lz2_in"], 2.0)
    c[0] *= 2.0
    c[nz - 1] *= 2.0
    c *= 0.5
    r = t.btran(c, "cff")
    err = np.abs(r - g["cheby_8x8x33_lz2_out"]).max()
    assert err <= 1e-14 * nx * ny * nz * 0.25
