"""SAR image formation by fast factorized back-projection, over the C ABI.

Mirrors the NFFT-interpolated branch of the reference's
``FFBP(data, a, b)`` (BP_FBP_FFBP/FFBP.m:1-29) and its recursion
``FFBP_POLAR_NFFT`` (FFBP_POLAR_NFFT.m:1-158): the image of pulses a..b
(1-based, inclusive, as in MATLAB) on the Cartesian scene points
``data["x_mat"], data["y_mat"], data["z_mat"]``.  The reference's globals
(c, fc, BW, f2) are keyword arguments.  Only the scene's polar coordinates
(FFBP.m:10-22) are formed here, on the host in FP64; the recursion, its Knab
regridding, the leaves' 1D NFFTs and every per-pixel pass run in
libnfft2d_gb300.so (nfft2d_ffbp_polar).  There is no CPU path.

``data`` holds, as the reference's struct: AntX, AntY, AntZ (Np antenna
positions), R0 (Np reference ranges), phdata (K x Np complex: column n is
pulse n's frequency samples) and x_mat, y_mat, z_mat.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check


def polar_grid(data: dict, a: int):
    """FFBP.m:10-20: range and direction cosine of every scene point seen
    from antenna a (1-based), the track direction taken towards antenna a+1."""
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


def FFBP_polar(data: dict, a: int, b: int, rho_out, cos_out, *, c: float, fc: float, BW: float, f2: float,
               precision: str = "f32", stream: torch.cuda.Stream | None = None, stats: dict | None = None
               ) -> torch.Tensor:
    """FFBP_POLAR_NFFT(data, a, b, 0) on given polar output points (len1 x len2
    FP64 arrays, host or device); returns the len1 x len2 complex image.  A
    dict passed as `stats` receives the work counts (nfft2d_ffbp_stats)."""
    lib = _lib.load()
    if precision not in ("f32", "f64"):
        raise ValueError("precision must be 'f32' or 'f64'")
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = stream if stream is not None else torch.cuda.current_stream()
    cdt = torch.complex64 if precision == "f32" else torch.complex128
    X, Y, Z, R0 = (np.ascontiguousarray(np.asarray(data[k], dtype=np.float64).ravel())
                   for k in ("AntX", "AntY", "AntZ", "R0"))
    ph = data["phdata"]
    ph = ph if isinstance(ph, torch.Tensor) else torch.from_numpy(np.asarray(ph))
    nf, npulse = ph.shape
    # pulse-major: column n of the reference's K x Np array is contiguous
    ph = ph.to(device=dev, dtype=cdt).T.contiguous()
    r = torch.as_tensor(rho_out, dtype=torch.float64, device=dev).contiguous()
    q = torch.as_tensor(cos_out, dtype=torch.float64, device=dev).contiguous()
    if r.dim() != 2 or r.shape != q.shape:
        raise ValueError("rho_out and cos_out must be equal-shape 2-D arrays")
    len1, len2 = r.shape
    image = torch.empty(len1, len2, dtype=cdt, device=dev)
    sar = _lib.Sar(float(c), float(fc), float(BW), float(f2))
    st = _lib.FfbpStats()
    dp = ctypes.c_void_p
    check(lib.nfft2d_ffbp_polar(ctypes.byref(sar), int(npulse), X.ctypes.data_as(dp), Y.ctypes.data_as(dp),
                                Z.ctypes.data_as(dp), R0.ctypes.data_as(dp), int(nf), dp(ph.data_ptr()), int(a) - 1,
                                int(b) - 1, int(len1), int(len2), dp(r.data_ptr()), dp(q.data_ptr()),
                                _lib.F32 if precision == "f32" else _lib.F64, dp(image.data_ptr()),
                                dp(stream.cuda_stream), ctypes.byref(st)), "nfft2d_ffbp_polar")
    if stats is not None:
        stats.update(st.as_dict())
    return image


def FFBP(data: dict, a: int, b: int, *, c: float, fc: float, BW: float, f2: float, precision: str = "f32",
         stream: torch.cuda.Stream | None = None, stats: dict | None = None) -> torch.Tensor:
    """FFBP.m:1-29 (NFFT-interpolated branch): the image of pulses a..b on the
    scene points data["x_mat"], data["y_mat"], data["z_mat"]."""
    rho, cosa = polar_grid(data, a)
    return FFBP_polar(data, a, b, rho, cosa, c=c, fc=fc, BW=BW, f2=f2, precision=precision, stream=stream,
                      stats=stats)


__all__ = ["FFBP", "FFBP_polar", "polar_grid"]
