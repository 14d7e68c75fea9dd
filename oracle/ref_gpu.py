"""The reference's own GPU spreading (NFFT/NFFT2_2D.cu, NFFT2_2D_GPU) as a
parity oracle -- TEST INFRASTRUCTURE ONLY.

``oracle/build_ref.py`` compiles the reference file unchanged (with the
stand-in headers of ``oracle/ref_shims``) into ``oracle/_ref/nfft2_2d_ref.cubin``
and the restated host side (``oracle/ref_harness.cpp``) into
``oracle/_ref/libref_harness.so``.  This module calls the harness on torch
CUDA tensors.  Only tests and bench.py's reference arm use it.

The reference computes, for x, y in grid units (period N1, N2), sigma = 2,
K = 6:
    result[i, j] = sum_p data_p exp(-2 pi i ((i - N1/2) x_p / N1 + (j - N2/2) y_p / N2))
with its float2 / double2 overloads.
"""
from __future__ import annotations

import ctypes
import os

from . import build_ref

_lib = None


def available() -> bool:
    """True when the device-linked reference cubin exists (it is built where
    the reference checkout is and travels as a file)."""
    return os.path.exists(build_ref.CUBIN)


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not available():
        raise RuntimeError("reference cubin missing: run oracle.build_ref.build() where the reference is checked out")
    build_ref.build_harness()
    lib = ctypes.CDLL(build_ref.HARNESS_LIB)
    lib.ref_last_error.restype = ctypes.c_char_p
    lib.ref_load.argtypes = [ctypes.c_char_p]
    for name, real in (("ref_nfft2_2d_gpu_f32", ctypes.c_void_p), ("ref_nfft2_2d_gpu_f64", ctypes.c_void_p)):
        fn = getattr(lib, name)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, real, real, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                       ctypes.c_longlong, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    rc = lib.ref_load(build_ref.CUBIN.encode())
    if rc != 0:
        raise RuntimeError(f"ref_load failed: {lib.ref_last_error().decode()}")
    _lib = lib
    return lib


def nfft2_2d_gpu(data, x, y, N1: int, N2: int, timing: bool = False):
    """Run the reference's NFFT2_2D_GPU on CUDA tensors (complex64 data with
    float32 x, y, or complex128 with float64) and return the N1 x N2 result.
    Inputs are copied into buffers padded to a multiple of 256 points (the
    reference reads them before its bounds guard).  With timing=True also
    returns (interpolation kernel ms by CUDA events, whole call ms by host
    clock)."""
    import torch

    lib = _load()
    M = int(x.numel())
    if M == 0 or y.numel() != M or data.numel() != M:
        raise ValueError("x, y and data need the same, non-zero length")
    dbl = data.dtype == torch.complex128
    rdt = torch.float64 if dbl else torch.float32
    cdt = torch.complex128 if dbl else torch.complex64
    m_alloc = ((M + 255) // 256) * 256
    dev = data.device
    xp = torch.zeros(m_alloc, dtype=rdt, device=dev)
    yp = torch.zeros(m_alloc, dtype=rdt, device=dev)
    dp = torch.zeros(m_alloc, dtype=cdt, device=dev)
    xp[:M] = x.reshape(-1).to(rdt)
    yp[:M] = y.reshape(-1).to(rdt)
    dp[:M] = data.reshape(-1).to(cdt)
    out = torch.zeros(N1, N2, dtype=cdt, device=dev)
    torch.cuda.synchronize(dev)
    t_int = ctypes.c_float(0.0)
    t_tot = ctypes.c_float(0.0)
    fn = lib.ref_nfft2_2d_gpu_f64 if dbl else lib.ref_nfft2_2d_gpu_f32
    rc = fn(out.data_ptr(), dp.data_ptr(), xp.data_ptr(), yp.data_ptr(), int(N1), int(N2), M, m_alloc,
            ctypes.byref(t_int), ctypes.byref(t_tot))
    if rc != 0:
        raise RuntimeError(f"reference NFFT2_2D_GPU failed ({rc}): {lib.ref_last_error().decode()}")
    if timing:
        return out, float(t_int.value), float(t_tot.value)
    return out
