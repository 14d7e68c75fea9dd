"""Generate tests/golden/nfft_golden.npz.

The reference ships no golden vectors and its MATLAB code cannot run here,
so the fixtures come from a numpy transliteration of the reference MATLAB
files, written independently of oracle/nfft2d_oracle.c (numpy's FFT instead
of the oracle's, scipy's I0 instead of the oracle's series, MATLAB's
column-major meshgrid/reshape semantics kept literally):

  * ndft2_2d_m   -- NFFT/NFFT2/Matlab/NDFT2_2D.m:1-16
  * nfft2_2d_m   -- NFFT/NFFT2/Matlab/NFFT2_2D.m:1-72 (c = 2, K = 6)
  * nfft1_2d_m   -- BP_FBP_FFBP/NFFT1_2D.m:1-69       (c = 2, K = 6)

Cases:
  * "reftest": the reference's own acceptance test, Test_NFFT2_2D.m:5-29 --
    121 points x = M_x*(lambda/2)*(rand-0.5) (M_x = M_y = 11, lambda = 1),
    complex data (rand-0.5) + 1i*(rand-0.5), NDFT2_2D(data, x, y, 22, 22) vs
    NFFT2_2D(data, y, x, 22, 22); the MATLAB rand is replaced by a seeded PCG64.
  * "fwd":  NFFT1_2D on a 16 x 16 complex grid at 50 points.
  * "rect": NFFT2_2D with M1 = 16, M2 = 24 at 80 points.

Run:  python tests/golden/make_golden.py   (writes the .npz next to this file)
"""
from __future__ import annotations

import os

import numpy as np
from scipy.special import i0

HERE = os.path.dirname(os.path.abspath(__file__))


def matlab_round(v):
    return np.where(v < 0, -np.floor(-v + 0.5), np.floor(v + 0.5))


def ndft2_2d_m(data, x, y, N, M):
    u = np.arange(-(N / 2), N / 2)                 # :3
    v = np.arange(-(M / 2), M / 2)                 # :4
    U, V = np.meshgrid(u, v)                       # :6   (M x N, like MATLAB)
    U = U.reshape(N * M, order="F")                # :8
    V = V.reshape(N * M, order="F")                # :9
    X, U2 = np.meshgrid(x, U)                      # :11
    Y, V2 = np.meshgrid(y, V)                      # :12
    Kern = np.exp(-1j * 2 * np.pi * X * U2 / N) * np.exp(-1j * 2 * np.pi * Y * V2 / N)  # :14
    return (Kern @ data).reshape(N, M, order="F")  # :16


def _phi_cap(x, c, K, alfa):
    mu = matlab_round(c * x)
    KK, MU = np.meshgrid(np.arange(-K, K + 1), mu)
    X = x[:, None] * np.ones((1, 2 * K + 1))
    P = np.sqrt((K ** 2 - (c * X - (MU + KK)) ** 2).astype(np.complex128))
    with np.errstate(invalid="ignore", divide="ignore"):
        ph = (1 / np.pi) * np.sinh(alfa * P) / P
    ph[P == 0] = alfa / np.pi
    return mu.astype(np.int64), ph.real


def nfft2_2d_m(data, x1, x2, M1, M2, c=2, K=6):
    alfa = (2 - 1 / c) * np.pi - 0.01                              # :8
    mu1, phi_cap1 = _phi_cap(x1, c, K, alfa)                        # :14-21
    mu2, phi_cap2 = _phi_cap(x2, c, K, alfa)                        # :23-27
    xi1 = 2 * np.pi * np.arange(-M1 / 2, M1 / 2) / (c * M1)          # :33-35
    phi1 = i0(K * np.sqrt(alfa ** 2 - xi1 ** 2))
    xi2 = 2 * np.pi * np.arange(-M2 / 2, M2 / 2) / (c * M2)          # :37-39
    phi2 = i0(K * np.sqrt(alfa ** 2 - xi2 ** 2))
    PHI2, PHI1 = np.meshgrid(phi2, phi1)                            # :41
    u = np.zeros((c * M1, c * M2), dtype=np.complex128)             # :47
    for k in range(len(data)):                                      # :48-56
        for l1 in range(-K, K + 1):
            p1 = np.mod(mu1[k] + l1 + M1 * c // 2, c * M1)
            p2 = np.mod(mu2[k] + np.arange(-K, K + 1) + M2 * c // 2, c * M2)
            u[p1, p2] += data[k] * phi_cap1[k, l1 + K] * phi_cap2[k, :]
    FFT_Mc = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(u)))      # :63
    a1, a2 = (c - 1) * M1 // 2, (c - 1) * M2 // 2
    return FFT_Mc[a1:a1 + M1, a2:a2 + M2] / (PHI1 * PHI2)           # :70


def nfft1_2d_m(data, x1, x2, c=2, K=6):
    N1, N2 = data.shape                                             # :3-4
    alfa = (2 - 1 / c) * np.pi - 0.01                              # :11
    xi1 = 2 * np.pi * np.arange(-N1 / 2, N1 / 2) / (c * N1)          # :17-22
    xi2 = 2 * np.pi * np.arange(-N2 / 2, N2 / 2) / (c * N2)
    phi1 = i0(K * np.sqrt(alfa ** 2 - xi1 ** 2))
    phi2 = i0(K * np.sqrt(alfa ** 2 - xi2 ** 2))
    PHI2, PHI1 = np.meshgrid(phi2, phi1)                            # :23
    mu1, sp1 = _phi_cap(x1, c, K, alfa)                             # :29-36
    mu2, sp2 = _phi_cap(x2, c, K, alfa)                             # :38-42
    u = np.zeros((c * N1, c * N2), dtype=np.complex128)             # :48
    a1, a2 = (c - 1) * N1 // 2, (c - 1) * N2 // 2
    u[a1:a1 + N1, a2:a2 + N2] = data / (PHI1 * PHI2)                # :49
    U = np.fft.fft2(np.fft.ifftshift(u))                            # :55
    res = np.zeros(len(x1), dtype=np.complex128)                    # :61
    for l in range(len(x1)):                                        # :62-67
        for m1 in range(-K, K + 1):
            rows = np.mod(mu1[l] + m1, c * N1)
            cols = np.mod(mu2[l] + np.arange(-K, K + 1), c * N2)
            res[l] += np.sum(sp1[l, m1 + K] * sp2[l, :] * U[rows, cols])
    return res


def main():
    rng = np.random.default_rng(20240601)
    out = {}
    # --- reference acceptance test (Test_NFFT2_2D.m:5-29)
    M_x = M_y = 11
    N = M = 22
    lam = 1.0
    x = M_x * (lam / 2) * (rng.random(M_x * M_y) - 0.5)
    y = M_y * (lam / 2) * (rng.random(M_x * M_y) - 0.5)
    data = (rng.random(M_x * M_y) - 0.5) + 1j * (rng.random(M_x * M_y) - 0.5)
    t1 = ndft2_2d_m(data, x, y, N, M)
    t2 = nfft2_2d_m(data, y, x, M, N)
    out.update(reftest_x=x, reftest_y=y, reftest_data=data, reftest_ndft=t1, reftest_nfft=t2,
               reftest_err_pct=100 * np.sqrt(np.sum(np.abs(t1 - t2) ** 2) / np.sum(np.abs(t1) ** 2)))
    # --- forward NFFT1_2D
    N1 = N2 = 16
    F = rng.standard_normal((N1, N2)) + 1j * rng.standard_normal((N1, N2))
    xf1 = (rng.random(50) - 0.5) * N1
    xf2 = (rng.random(50) - 0.5) * N2
    out.update(fwd_F=F, fwd_x1=xf1, fwd_x2=xf2, fwd_out=nfft1_2d_m(F, xf1, xf2))
    # --- rectangular NFFT2_2D
    d = rng.standard_normal(80) + 1j * rng.standard_normal(80)
    xr1 = (rng.random(80) - 0.5) * 16
    xr2 = (rng.random(80) - 0.5) * 24
    out.update(rect_d=d, rect_x1=xr1, rect_x2=xr2, rect_out=nfft2_2d_m(d, xr1, xr2, 16, 24))
    path = os.path.join(HERE, "nfft_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}; reference-test NFFT vs NDFT error {float(out['reftest_err_pct']):.3e} %")


if __name__ == "__main__":
    main()
