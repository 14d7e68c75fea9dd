"""Type-3 2D NUFFT (nonuniform points to nonuniform frequencies), over the
C ABI.

Mirrors ``NUFFT_2D_CPU(x, y, s, t, f, F, eps, len_in, len_out)``
(NFFT/NFFT3/C/NFFT3_2D_C.h, NFFT3_2D_C.cpp:199-312) and its MATLAB gateway
``F = NFFT3_2D_C_mex(x, y, s, t, f, eps)``:
    F[k] = sum_j f[j] exp(-i (s[k] x[j] + t[k] y[j]))
by Gaussian gridding (nfft2d_nufft3_2d).  There is no CPU path.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import check


def NUFFT_2D(x, y, s, t, f, eps: float, precision: str | None = None,
             stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    """x, y: len_in points; s, t: len_out frequencies (any real values, FP64
    on the device); f: len_in complex values (complex64 -> FP32 grid,
    complex128 -> FP64).  Returns F (len_out complex, f's dtype)."""
    lib = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = stream if stream is not None else torch.cuda.current_stream()
    f = torch.as_tensor(f, device=dev)
    if precision is None:
        precision = "f32" if f.dtype == torch.complex64 else "f64"
    cdt = torch.complex64 if precision == "f32" else torch.complex128
    f = f.to(cdt).contiguous().reshape(-1)
    x, y, s, t = (torch.as_tensor(v, dtype=torch.float64, device=dev).contiguous().reshape(-1) for v in (x, y, s, t))
    if x.numel() != f.numel() or y.numel() != f.numel() or s.numel() != t.numel():
        raise ValueError("x, y and f need one entry per point; s and t one per frequency")
    F = torch.empty(s.numel(), dtype=cdt, device=dev)
    p = ctypes.c_void_p
    check(lib.nfft2d_nufft3_2d(p(x.data_ptr()), p(y.data_ptr()), p(s.data_ptr()), p(t.data_ptr()), p(f.data_ptr()),
                               p(F.data_ptr()), float(eps), f.numel(), s.numel(),
                               _lib.F32 if precision == "f32" else _lib.F64, p(stream.cuda_stream)),
          "nfft2d_nufft3_2d")
    return F


__all__ = ["NUFFT_2D"]
