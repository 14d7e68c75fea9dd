"""CPU restatement of the reference's FFBP image formation -- TEST
INFRASTRUCTURE ONLY (the checker of miscellaneous_gb300.sar).

Follows, step by step, the NFFT-interpolated branch of
  BP_FBP_FFBP/FFBP.m:1-29              (scene -> polar grid of antenna a),
  BP_FBP_FFBP/FFBP_POLAR_NFFT.m:1-158  (recursion and knabNFFT2D regridding),
  BP_FBP_FFBP/BP_POLAR_NFFT.m:1-25     (leaf back-projection through NFFT1_1D),
with the C restatements of knabNFFT2D.m and NFFT1_1D.m (oracle.knab_nfft2d,
oracle.nfft1_1d).  FP64 throughout; pulses are 1-based as in MATLAB.

Two expressions are written in the IEEE form both this restatement and the
library evaluate bit for bit (sizes and axes of every level depend on them):
cos(atan2(y, x)) (FFBP_POLAR_NFFT.m:46) as x / sqrt(x^2 + y^2), equal within
an ulp or two; mean(diff(v)) as the differences summed in index order.
"""
from __future__ import annotations

import math

import numpy as np

from . import knab_nfft2d, nfft1_1d


def linspace(d1: float, d2: float, n: int) -> np.ndarray:
    """MATLAB linspace(d1, d2, n): d1 + i (d2 - d1)/(n - 1), the last sample d2."""
    step = (d2 - d1) / (n - 1)
    v = d1 + np.arange(n, dtype=np.float64) * step
    v[-1] = d2
    return v


def mean_diff(v: np.ndarray) -> float:
    s = 0.0
    for i in range(v.size - 1):
        s += float(v[i + 1] - v[i])
    return s / (v.size - 1)


def _dist(data, i: int, j: int) -> float:
    """sqrt((AntX(i) - AntX(j))^2 + ...) for 1-based pulses."""
    dx = data["AntX"][i - 1] - data["AntX"][j - 1]
    dy = data["AntY"][i - 1] - data["AntY"][j - 1]
    dz = data["AntZ"][i - 1] - data["AntZ"][j - 1]
    return math.sqrt(dx * dx + dy * dy + dz * dz)


def bp_polar_nfft(data, sar, minInd: int, maxInd: int, pho, cosa):
    """BP_POLAR_NFFT.m:1-25 on points (pho, cosa)."""
    c, fc, BW = sar["c"], sar["fc"], sar["BW"]
    im = np.zeros(pho.size, dtype=np.complex128)
    for n in range(minInd, maxInd + 1):                                   # :11
        xsi = _dist(data, n, minInd)                                      # :14
        delta_r = np.sqrt(pho * pho + xsi * xsi - 2.0 * pho * xsi * cosa) - data["R0"][n - 1]  # :15
        pc = np.exp(1j * (4.0 * math.pi * fc * delta_r / c))              # :17
        im = im + pc.ravel() * nfft1_1d(data["phdata"][:, n - 1], ((-2.0 * BW) / c * delta_r).ravel())  # :19
    return im.reshape(pho.shape)                                          # :23


def ffbp_polar_nfft(data, sar, a: int, b: int, rho_out, cos_out):
    """FFBP_POLAR_NFFT.m:1-158 (the knabNFFT image only)."""
    c, fc, BW, f2 = sar["c"], sar["fc"], sar["BW"], sar["f2"]
    center = (a + b) // 2                                                 # :24
    if b - a <= 2:                                                        # :27-36
        return bp_polar_nfft(data, sar, a, b, rho_out, cos_out)
    sin_out = np.sqrt(1.0 - cos_out * cos_out)                            # :39
    k4c = 4.0 * math.pi / c
    out = None
    for sa, sb, ref, L in ((a, center, a, _dist(data, center, a)),       # :44, :54
                           (center + 1, b, center + 1, _dist(data, b, center))):  # :96, :106
        dist = _dist(data, ref, a)
        x = rho_out * cos_out - dist
        y = rho_out * sin_out
        rho_i = np.sqrt(x * x + y * y)                                    # :45
        with np.errstate(invalid="ignore", divide="ignore"):
            cos_i = np.where(rho_i > 0, x / rho_i, 1.0)                   # :46
        maxrho, minrho = float(rho_i.max()), float(rho_i.min())           # :49-52
        maxcos, mincos = float(cos_i.max()), float(cos_i.min())
        Nrho = math.floor((maxrho - minrho) / (c / (2.0 * BW))) * 5.0     # :58
        Ncos = math.floor((maxcos - mincos) / (c / (2.0 * f2 * L))) * 5.0 + 3.0  # :59
        tr = 30.0 * (maxrho - minrho) / (Nrho - 1.0)
        tc = 30.0 * (maxcos - mincos) / (Ncos - 1.0)
        rho_in = linspace(minrho - tr, maxrho + tr, int(Nrho) + 60)        # :63
        cos_in = linspace(mincos - tc, maxcos + tc, int(Ncos) + 60)        # :64
        RHO_IN, COS_IN = np.meshgrid(rho_in, cos_in)                       # :66
        sub = ffbp_polar_nfft(data, sar, sa, sb, RHO_IN, COS_IN)           # :71
        sub = sub * np.exp(-1j * ((k4c * RHO_IN) * fc))                    # :73-79
        B1 = (1.0 / mean_diff(rho_in)) * 0.5                               # :81, :89
        B2 = (1.0 / mean_diff(cos_in)) * 0.5
        rec, _ = knab_nfft2d(complex(float("nan"), 0.0), rho_in, cos_in, sub, rho_i, cos_i, B1, B2)  # :89
        rec = rec * np.exp(1j * ((k4c * rho_i) * fc))
        out = rec if out is None else out + rec                           # :152
    return out


def polar_grid(data, a: int):
    """FFBP.m:10-20."""
    i = a - 1
    X, Y, Z = (np.asarray(data[k], dtype=np.float64).ravel() for k in ("AntX", "AntY", "AntZ"))
    Dx, Dy, Dz = X[i + 1] - X[i], Y[i + 1] - Y[i], Z[i + 1] - Z[i]
    nrm = np.sqrt(Dx ** 2 + Dy ** 2 + Dz ** 2)
    dx, dy, dz = Dx / nrm, Dy / nrm, Dz / nrm
    x = np.asarray(data["x_mat"], dtype=np.float64)
    y = np.asarray(data["y_mat"], dtype=np.float64)
    z = np.asarray(data["z_mat"], dtype=np.float64)
    rho = np.sqrt((x - X[i]) ** 2 + (y - Y[i]) ** 2 + (z - Z[i]) ** 2)
    cosa = (x - X[i]) / rho * dx + (y - Y[i]) / rho * dy + (z - Z[i]) / rho * dz
    return rho, cosa


def ffbp(data, sar, a: int, b: int):
    """FFBP.m:1-29 (knabNFFT image)."""
    rho, cosa = polar_grid(data, a)
    return ffbp_polar_nfft(data, sar, a, b, rho, cosa)


def point_target_scene(Np: int = 16, nf: int = 64, Nx: int = 32, step: float = 0.08, R: float = 10e3,
                       dep: float = math.pi / 6, maxAz: float = 3 * math.pi / 180, targets=((0.0, 0.0),),
                       fc: float = 10e9, BW: float = 600e6):
    """The reference's synthetic scenario (BP_FBP_FFBP_main.m:7-103) at a
    chosen size: a straight track at range R and depression dep, Np pulses
    over maxAz, nf frequency samples over BW around fc, an Nx x Nx scene with
    the given pixel step, and unit point targets at (x, y) on z = 0."""
    c = 299792458.0
    deltaF = BW / nf
    minF = fc - BW / 2.0
    f2 = minF + nf * deltaF
    az = np.arange(Np) / Np * maxAz - maxAz / 2
    X = R * math.cos(dep) * np.ones(Np)
    Y = R * math.cos(dep) * np.tan(az)
    Z = R * math.sin(dep) * np.ones(Np)
    R0 = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    W = Nx * step
    v = np.linspace(-W / 2, W / 2, Nx)
    x_mat, y_mat = np.meshgrid(v, v)
    ph = np.zeros((nf, Np), dtype=np.complex128)
    fk = minF + np.arange(nf) * deltaF
    for tx, ty in targets:
        dR = np.sqrt((X - tx) ** 2 + (Y - ty) ** 2 + Z ** 2) - R0
        ph += np.exp(-1j * 4 * math.pi * np.outer(fk, dR) / c)
    data = dict(AntX=X, AntY=Y, AntZ=Z, R0=R0, phdata=ph, x_mat=x_mat, y_mat=y_mat, z_mat=np.zeros_like(x_mat))
    sar = dict(c=c, fc=fc, BW=BW, f2=f2)
    return data, sar
