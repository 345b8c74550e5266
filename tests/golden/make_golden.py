"""Generates tests/golden/known_answers.npz: inputs and closed-form expected
outputs of the reference sample programs' analytic checks (no FFT is used to
make them).

    python tests/golden/make_golden.py

* sine_*      driver_sine.F90:322-355: A = sin(2 pi x/nx) sin(2 pi y/ny)
              sin(2 pi z/nz); each factor has -i n/2 at k = 1 and +i n/2 at
              k = n-1, so the r2c spectrum has 4 stored non-zeros of +-N/8 i^3.
* spikes_*    driver_inverse.F90: the complex wave e^{2 pi i kx/nx}
              sin(2 pi 2 ky/ny) sin(2 pi 3 kz/nz) through 'tff' gives +-N/4 at
              four points (init_wave2 / the sample's expected values).
* dct_*       'ffc' of cos(2 pi x/nx) cos(pi m z/(nz-1)): REDFT00 of one
              cosine is nz-1 at k = m, so B(1, 0, m) = nx/2 ny (nz-1).
* dst_*       'ffs' of cos(2 pi x/nx) sin(pi (m+1)(z+1)/(nz+1)): RODFT00 of
              one sine is nz+1 at k = m, so B(1, 0, m) = nx/2 ny (nz+1).
* cheby_*     driver_cheby.F90:96-111,218-284: d/dz sin(z) on the
              Gauss-Lobatto points z_j = cos(pi j/(nz-1)) 2/Lz is cos(z).
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def sine(nx, ny, nz):
    tp = 8 * np.arctan(1.0)
    a = (np.sin(np.arange(nz) * tp / nz)[:, None, None] * np.sin(np.arange(ny) * tp / ny)[None, :, None]
         * np.sin(np.arange(nx) * tp / nx)[None, None, :])

    def ax(n, k):
        return np.where(k == 1, -0.5j * n, np.where(k == n - 1, 0.5j * n, 0))

    b = (ax(nz, np.arange(nz))[:, None, None] * ax(ny, np.arange(ny))[None, :, None]
         * ax(nx, np.arange(nx // 2 + 1))[None, None, :])
    return a, b


def spikes(nx, ny, nz):
    tp = 8 * np.arctan(1.0)
    x = np.arange(nx // 2 + 1)
    wave = ((np.cos(x * tp / nx) + 1j * np.sin(x * tp / nx))[None, None, :]
            * np.sin(np.arange(ny) * 2.0 * tp / ny)[None, :, None]
            * np.sin(np.arange(nz) * 3.0 * tp / nz)[:, None, None])
    n = nx * ny * nz
    r = np.zeros((nz, ny, nx))
    r[3, 2, nx - 1] = -n * 0.25
    r[nz - 3, 2, nx - 1] = n * 0.25
    r[3, ny - 2, nx - 1] = n * 0.25
    r[nz - 3, ny - 2, nx - 1] = -n * 0.25
    return wave, r


def dct(nx, ny, nz, m):
    tp = 8 * np.arctan(1.0)
    a = np.cos(np.arange(nx) * tp / nx)[None, None, :] * np.cos(np.pi * m * np.arange(nz) / (nz - 1))[:, None, None]
    a = np.broadcast_to(a, (nz, ny, nx)).copy()
    b = np.zeros((nz, ny, nx // 2 + 1), dtype=np.complex128)
    b[m, 0, 1] = nx / 2 * ny * (nz - 1)
    return a, b


def dst(nx, ny, nz, m):
    tp = 8 * np.arctan(1.0)
    a = (np.cos(np.arange(nx) * tp / nx)[None, None, :]
         * np.sin(np.pi * (m + 1) * (np.arange(nz) + 1) / (nz + 1))[:, None, None])
    a = np.broadcast_to(a, (nz, ny, nx)).copy()
    b = np.zeros((nz, ny, nx // 2 + 1), dtype=np.complex128)
    b[m, 0, 1] = nx / 2 * ny * (nz + 1)
    return a, b


def cheby(nx, ny, nz, lz):
    zc = np.cos(np.pi * np.arange(nz) / (nz - 1)) * 2.0 / lz
    a = np.broadcast_to(np.sin(zc)[:, None, None], (nz, ny, nx)).copy()
    d = np.broadcast_to(np.cos(zc)[:, None, None], (nz, ny, nx)).copy()
    return a, d


def main():
    out = {}
    for shape in [(14, 26, 38), (16, 12, 10)]:
        a, b = sine(*shape)
        tag = "x".join(map(str, shape))
        out[f"sine_{tag}_in"], out[f"sine_{tag}_out"] = a, b
    w, r = spikes(16, 16, 16)
    out["spikes_16x16x16_in"], out["spikes_16x16x16_out"] = w, r
    a, b = dct(12, 8, 17, 5)
    out["dct_12x8x17_m5_in"], out["dct_12x8x17_m5_out"] = a, b
    a, b = dst(12, 8, 15, 4)
    out["dst_12x8x15_m4_in"], out["dst_12x8x15_m4_out"] = a, b
    a, d = cheby(8, 8, 33, 2.0)
    out["cheby_8x8x33_lz2_in"], out["cheby_8x8x33_lz2_out"] = a, d
    np.savez_compressed(os.path.join(HERE, "known_answers.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
