"""Generate tests/golden/nfft_golden.npz.

The reference ships no golden vectors and its MATLAB code cannot run here,
so the fixtures come from a numpy transliteration of the reference MATLAB
files, written independently of oracle/nfft2d_oracle.c (numpy's FFT instead
of the oracle's, scipy's I0 instead of the oracle's series, MATLAB's
column-major meshgrid/reshape semantics kept literally):

  * ndft2_2d_m   -- NFFT/NFFT2/Matlab/NDFT2_2D.m:1-16
  * nfft2_2d_m   -- NFFT/NFFT2/Matlab/NFFT2_2D.m:1-72 (c = 2, K = 6)
  * nfft1_2d_m   -- BP_FBP_FFBP/NFFT1_2D.m:1-69       (c = 2, K = 6)
  * knab_window_m  -- BP_FBP_FFBP/KnabWindow.m:11-47 with ConvWindow.m and
                      IntervalIntersection.m (scipy's QUADPACK quad in place
                      of MATLAB's adaptive Simpson quad, both at 1e-12)
  * knab_nfft2d_m  -- BP_FBP_FFBP/knabNFFT2D.m:1-79 with
                      NFFT_Based_Selvas_Approach_for_Signal_Interp_2D.m:4-28

Cases:
  * "reftest": the reference's own acceptance test, Test_NFFT2_2D.m:5-29 --
    121 points x = M_x*(lambda/2)*(rand-0.5) (M_x = M_y = 11, lambda = 1),
    complex data (rand-0.5) + 1i*(rand-0.5), NDFT2_2D(data, x, y, 22, 22) vs
    NFFT2_2D(data, y, x, 22, 22); the MATLAB rand is replaced by a seeded PCG64.
  * "fwd":  NFFT1_2D on a 16 x 16 complex grid at 50 points.
  * "rect": NFFT2_2D with M1 = 16, M2 = 24 at 80 points.
  * knab_golden.npz: knabNFFT2D on a 20 x 24 raster (rows: cos(alpha),
    columns: rho) to a 14 x 33 output raster, rotated slightly so the
    output points are not separable, with one column and one row outside
    the input range (extrapolation value); and KnabWindow at (T, B, P, N) =
    (0.25, 1.8, 18, 24).  B is chosen so that floor() in KnabWindow.m:19 and
    round() in knabNFFT2D.m:45-46 are far from a tie.

Run:  python tests/golden/make_golden.py   (writes the .npz files next to this file)
"""
from __future__ import annotations

import os

import numpy as np
from scipy.integrate import quad
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


def conv_window_m(f, B, T):
    f = np.atleast_1d(np.asarray(f, dtype=np.float64))
    W = np.zeros(f.shape)                                                     # ConvWindow.m:7
    I = np.abs(f) < B / 2                                                     # :9
    den = B * np.real(np.sinc(1j * B * T / 2))
    W[I] = i0(np.pi * B * (T / 2) * np.sqrt(1 - (2 * f[I] / B) ** 2)) / den   # :11
    return W


def interval_intersection_m(IA, IB):
    if IA[1] < IB[0] or IB[1] < IA[0]:                                        # IntervalIntersection.m:6
        return None
    if IB[1] < IA[1]:                                                         # :13
        return [IA[0], IB[1]]
    return [IB[0], IA[1]]                                                     # :20


def knab_window_m(T, B, P, N):
    df = 1 / (N * T)                                                          # KnabWindow.m:16
    kg = int(np.floor((1 / T - B / 2) / df))                                  # :19
    f = -df * kg + df * np.arange(0, kg + 1)                                  # :22
    B0 = 1 / T                                                                # :24
    B1 = B0 - B                                                               # :25
    I = B1 / 2 <= (f + B0 / 2)                                                # :26
    G = np.zeros(2 * kg + 1)                                                  # :29
    G[:kg + 1][I] = 1                                                         # :32
    notI = np.nonzero(~I)[0]
    for k in range(notI[-1] + 1 if notI.size else 0):                        # :36
        IInt = interval_intersection_m([-B1 / 2, B1 / 2], f[k] + np.array([-B0 / 2, B0 / 2]))
        if IInt is not None:
            G[k] = quad(lambda x: conv_window_m(x, B1, 2 * P * T)[0], IInt[0], IInt[1],
                        epsabs=1e-12, epsrel=0, limit=500)[0]                 # :40
    G = G + G[::-1]                                                           # :45
    G[kg] -= 1                                                                # :46
    return G / N, kg                                                          # :47


def selva_interp_2d_m(INPUT_DATA, T1, T2, a, b, G, kgn, kgm, RHO_OUT_SHIFTED, COSALPHA_OUT_SHIFTED):
    N, M = INPUT_DATA.shape                                                   # Interp_2D.m:6-7
    sF = np.fft.fft2(INPUT_DATA)                                              # :9
    sF = sF[np.ix_(np.mod(np.arange(-kgn, kgn + 1), N), np.mod(np.arange(-kgm, kgm + 1), M))]  # :10
    sF = sF * G * (N * a) * (M * b)                                           # :11
    csF = sF.shape[0]
    if (b * M) % 2 == 0:                                                      # :14-18
        sF = np.hstack([np.zeros((csF, M * b // 2 - kgm)), sF, np.zeros((csF, M * b // 2 - kgm - 1))])
    else:
        sF = np.hstack([np.zeros((csF, (M * b - 2 * kgm - 1) // 2)), sF, np.zeros((csF, (M * b - 2 * kgm - 1) // 2))])
    rsF = sF.shape[1]
    if (a * N) % 2 == 0:                                                      # :21-25
        sF = np.vstack([np.zeros((N * a // 2 - kgn, rsF)), sF, np.zeros((N * a // 2 - kgn - 1, rsF))])
    else:
        sF = np.vstack([np.zeros(((N * a - 2 * kgn - 1) // 2, rsF)), sF, np.zeros(((N * a - 2 * kgn - 1) // 2, rsF))])
    x1 = (RHO_OUT_SHIFTED / (T1 / a)).reshape(-1, order="F")                  # :28
    x2 = (COSALPHA_OUT_SHIFTED / (T2 / b)).reshape(-1, order="F")
    return (1 / (a * b * N * M)) * np.conj(nfft1_2d_m(np.conj(sF), x1, x2))


def knab_nfft2d_m(ExtrapVal, RHO_IN, COSALPHA_IN, INPUT_DATA, RHO_OUT, COSALPHA_OUT, B1, B2):
    T1 = np.mean(np.diff(RHO_IN[0, :]))                                       # knabNFFT2D.m:6
    T2 = np.mean(np.diff(COSALPHA_IN[:, 0]))                                  # :7
    RHO_OUT_SHIFTED = RHO_OUT - RHO_IN.flat[0]                                # :23
    COSALPHA_OUT_SHIFTED = COSALPHA_OUT - COSALPHA_IN.flat[0]                 # :24
    len1, len2 = RHO_OUT_SHIFTED.shape                                        # :26-27
    N = (RHO_OUT_SHIFTED.max() - RHO_OUT_SHIFTED.min()) / (T1 * (1 - 1 / len2))           # :34
    M = (COSALPHA_OUT_SHIFTED.max() - COSALPHA_OUT_SHIFTED.min()) / (T2 * (1 - 1 / len1))  # :35
    if N < 1 or np.isnan(N):
        N = 1
    if M < 1 or np.isnan(M):
        M = 1
    a = int(matlab_round(len2 / N))                                           # :45
    b = int(matlab_round(len1 / M))                                           # :46
    if a < 2:                                                                 # :48-53
        a = 2
        ii = max(int(matlab_round(a * N)) - RHO_OUT_SHIFTED.shape[1], 0)
        RHO_OUT_SHIFTED = np.hstack([RHO_OUT_SHIFTED, np.zeros((RHO_OUT_SHIFTED.shape[0], ii))])
        COSALPHA_OUT_SHIFTED = np.hstack([COSALPHA_OUT_SHIFTED, np.zeros((COSALPHA_OUT_SHIFTED.shape[0], ii))])
    if b < 2:                                                                 # :55-60
        b = 2
        ii = max(int(matlab_round(b * M)) - RHO_OUT_SHIFTED.shape[0], 0)
        RHO_OUT_SHIFTED = np.vstack([RHO_OUT_SHIFTED, np.zeros((ii, RHO_OUT_SHIFTED.shape[1]))])
        COSALPHA_OUT_SHIFTED = np.vstack([COSALPHA_OUT_SHIFTED, np.zeros((ii, COSALPHA_OUT_SHIFTED.shape[1]))])
    P = 18                                                                    # :63
    Gn, kgn = knab_window_m(T1, B1, P, INPUT_DATA.T.shape[0])                 # :64
    Gm, kgm = knab_window_m(T2, B2, P, INPUT_DATA.T.shape[1])                 # :65
    Y, X = np.meshgrid(Gm, Gn)                                                # :66
    G = X * Y                                                                 # :67
    res = selva_interp_2d_m(INPUT_DATA.T, T1, T2, a, b, G, kgn, kgm, RHO_OUT_SHIFTED, COSALPHA_OUT_SHIFTED)
    result = res.reshape(RHO_OUT_SHIFTED.shape[0], COSALPHA_OUT_SHIFTED.shape[1], order="F")  # :71
    result = result[:len1, :len2]                                             # :72
    xout = (RHO_OUT[0, :] < RHO_IN[0, :].min()) | (RHO_OUT[0, :] > RHO_IN[0, :].max())              # :75
    yout = (COSALPHA_OUT[:, 0] < COSALPHA_IN[:, 0].min()) | (COSALPHA_OUT[:, 0] > COSALPHA_IN[:, 0].max())
    result[:, xout] = ExtrapVal                                               # :77
    result[yout, :] = ExtrapVal                                               # :78
    return result, dict(a=a, b=b, kgn=kgn, kgm=kgm)


def knab_case(seed=20240602):
    rng = np.random.default_rng(seed)
    Nrows, Ncols = 20, 24
    T1, T2 = 0.25, 0.02
    rho_in = 50.0 + T1 * np.arange(Ncols)
    cos_in = -0.2 + T2 * np.arange(Nrows)
    RHO_IN, COSALPHA_IN = np.meshgrid(rho_in, cos_in)
    data = rng.standard_normal((Nrows, Ncols)) + 1j * rng.standard_normal((Nrows, Ncols))
    len1, len2 = 14, 33
    r = np.linspace(rho_in[2], rho_in[-3], len2)
    c = np.linspace(cos_in[2], cos_in[-3], len1)
    Rg, Cg = np.meshgrid(r, c)
    # slight rotation (in sample units) so the output points are not separable
    u, v = (Rg - rho_in[0]) / T1, (Cg - cos_in[0]) / T2
    th = 0.05
    RHO_OUT = rho_in[0] + T1 * (np.cos(th) * u - np.sin(th) * v * 0.3)
    COSALPHA_OUT = cos_in[0] + T2 * (np.sin(th) * u * 0.3 + np.cos(th) * v)
    RHO_OUT[:, 0] = rho_in[0] - 0.4      # one column below the input range
    COSALPHA_OUT[-1, :] = cos_in[-1] + 0.03  # one row above it
    B1, B2 = 1.8, 17.0                   # 0.45 / T1 and 0.34 / T2
    ev = 0.25 - 0.5j
    out, info = knab_nfft2d_m(ev, RHO_IN, COSALPHA_IN, data, RHO_OUT, COSALPHA_OUT, B1, B2)
    G, kg = knab_window_m(0.25, 1.8, 18, 24)
    return dict(rho_in=rho_in, cos_in=cos_in, data=data, rho_out=RHO_OUT, cos_out=COSALPHA_OUT, B1=B1, B2=B2,
                extrap=ev, out=out, a=info["a"], b=info["b"], kgn=info["kgn"], kgm=info["kgm"],
                window_G=G, window_kg=kg)


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
    kpath = os.path.join(HERE, "knab_golden.npz")
    kc = knab_case()
    np.savez_compressed(kpath, **kc)
    print(f"wrote {kpath}; a = {kc['a']}, b = {kc['b']}, kgn = {kc['kgn']}, kgm = {kc['kgm']}")


if __name__ == "__main__":
    main()
