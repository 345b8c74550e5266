"""Index rules of the X passes' fused first FFT stage, restated on the host
(no GPU) and checked against numpy's real transforms:

* r2c: two real lines x1, x2 taken as one complex line z = x1 + i x2; after
  the complex FFT, X1[k] = (Z[k] + conj Z[N-k]) / 2 and
  X2[k] = -i (Z[k] - conj Z[N-k]) / 2 for k <= N/2;
* c2r: the pair's half spectra (N/2+1 modes) extended to a full line as
  z[p] = X1[p] + i X2[p], with X[p] = conj X[N-p] above N/2 (the mirror index
  the first stage reads) and the imaginary parts of the p = 0 and p = N/2
  modes ignored, as a c2r transform does; the inverse complex FFT then holds
  x1 in its real part and x2 in its imaginary part.

Even and odd N, including lengths whose first radix is 3 or 5."""
import numpy as np
import pytest


def _extend(X1, X2, N):
    """The c2r first-stage rule, point by point."""
    z = np.empty(N, dtype=np.complex128)
    for p in range(N):
        mir = 2 * p > N
        pm = N - p if mir else p
        x1, x2 = X1[pm], X2[pm]
        if pm == 0 or 2 * pm == N:
            x1, x2 = complex(x1.real, 0.0), complex(x2.real, 0.0)
        if mir:
            x1, x2 = np.conj(x1), np.conj(x2)
        z[p] = x1 + 1j * x2
    return z


@pytest.mark.parametrize("N", [2, 3, 5, 8, 12, 15, 16, 45, 64, 96, 100, 768 // 8])
def test_c2r_extension_matches_irfft(N):
    rng = np.random.default_rng(N)
    nh = N // 2 + 1
    X1 = rng.standard_normal(nh) + 1j * rng.standard_normal(nh)
    X2 = rng.standard_normal(nh) + 1j * rng.standard_normal(nh)
    z = np.fft.ifft(_extend(X1, X2, N)) * N  # unnormalised backward transform
    np.testing.assert_allclose(z.real, np.fft.irfft(X1, N) * N, atol=1e-12 * N)
    np.testing.assert_allclose(z.imag, np.fft.irfft(X2, N) * N, atol=1e-12 * N)


@pytest.mark.parametrize("N", [2, 3, 5, 8, 12, 15, 16, 45, 64, 96, 100])
def test_r2c_split_matches_rfft(N):
    rng = np.random.default_rng(100 + N)
    x1, x2 = rng.standard_normal(N), rng.standard_normal(N)
    Z = np.fft.fft(x1 + 1j * x2)
    k = np.arange(N // 2 + 1)
    Zc = np.conj(Z[(N - k) % N])
    np.testing.assert_allclose((Z[k] + Zc) / 2, np.fft.rfft(x1), atol=1e-12 * N)
    np.testing.assert_allclose(-1j * (Z[k] - Zc) / 2, np.fft.rfft(x2), atol=1e-12 * N)


def test_mirror_index_of_the_first_stage():
    # butterfly j of a radix-R first stage reads points p = j + q N/R; for
    # p > N/2 it reads mode N - p, never beyond N/2
    for N, R in ((1024, 8), (768, 8), (540, 4), (45, 3), (25, 5)):
        for j in range(N // R):
            for q in range(R):
                p = j + q * (N // R)
                pm = N - p if 2 * p > N else p
                assert 0 <= pm <= N // 2
