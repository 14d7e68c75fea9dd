"""Knab-window band-limited regridding on the GPU, over the C ABI.

Mirrors ``knabNFFT2D(ExtrapVal, RHO_IN, COSALPHA_IN, INPUT_DATA, RHO_OUT,
COSALPHA_OUT, B1, B2)`` (BP_FBP_FFBP/knabNFFT2D.m:1) -- same argument
meaning, same layout (INPUT_DATA rows <-> cos alpha, columns <-> rho), same
oversampling detection, window (KnabWindow.m, P = 18) and extrapolation
value -- and ``KnabWindow(T, B, P, N)`` (BP_FBP_FFBP/KnabWindow.m:11).

The raster FFT, the windowed zero-padded spectrum, the NFFT and the
extrapolation fill all run in libnfft2d_gb300.so; there is no CPU path.
``Regridder`` keeps the plan and the output points for repeated use (the
FFBP recursion regrids many rasters onto the same output grid).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def KnabWindow(T: float, B: float, P: int, N: int):
    """KnabWindow.m:11-47: returns (G, kg), G over frequencies -kg..kg
    (host FP64; needs no GPU)."""
    lib = _lib.load()
    kg = ctypes.c_int()
    check(lib.nfft2d_knab_window(float(T), float(B), int(P), int(N), None, 0, ctypes.byref(kg)),
          "nfft2d_knab_window")
    G = np.zeros(2 * kg.value + 1)
    check(lib.nfft2d_knab_window(float(T), float(B), int(P), int(N), G.ctypes.data_as(ctypes.c_void_p), G.size,
                                 ctypes.byref(kg)), "nfft2d_knab_window")
    return G, kg.value


def _axis(v, name: str, along_rows: bool) -> np.ndarray:
    """RHO_IN / COSALPHA_IN may be vectors or meshgrid matrices
    (knabNFFT2D.m:6-12): rho varies along a row, cos alpha along a column."""
    a = v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 2:
        a = a[:, 0] if along_rows else a[0, :]
    if a.ndim != 1:
        raise ValueError(f"{name} must be a vector or a meshgrid matrix")
    return np.ascontiguousarray(a)


class Regridder:
    """knabNFFT2D for one input raster geometry (Nrows x Ncols, axes rho_in
    and cos_in, bandwidths B1, B2) and one set of output points."""

    def __init__(self, rho_in, cos_in, B1: float, B2: float, precision: str = "f32",
                 stream: torch.cuda.Stream | None = None):
        self._lib = _lib.load()
        if precision not in ("f32", "f64"):
            raise ValueError("precision must be 'f32' or 'f64'")
        self.rho_in = _axis(rho_in, "RHO_IN", along_rows=False)
        self.cos_in = _axis(cos_in, "COSALPHA_IN", along_rows=True)
        self.Ncols, self.Nrows = self.rho_in.size, self.cos_in.size
        self.precision = precision
        self.cdtype = torch.complex64 if precision == "f32" else torch.complex128
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        h = ctypes.c_void_p()
        check(self._lib.nfft2d_knab_create(
            ctypes.byref(h), self.Nrows, self.Ncols, self.rho_in.ctypes.data_as(ctypes.c_void_p),
            self.cos_in.ctypes.data_as(ctypes.c_void_p), float(B1), float(B2),
            _lib.F32 if precision == "f32" else _lib.F64, ctypes.c_void_p(self.stream.cuda_stream)),
            "nfft2d_knab_create")
        self._h = h
        self.shape = None
        self._keep = ()

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.nfft2d_knab_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_points(self, rho_out: torch.Tensor, cos_out: torch.Tensor) -> None:
        """Output coordinates: len1 x len2 CUDA tensors (float32 or float64)."""
        if rho_out.shape != cos_out.shape or rho_out.dim() != 2:
            raise ValueError("RHO_OUT and COSALPHA_OUT must be equal-shape 2-D tensors")
        if rho_out.dtype not in (torch.float32, torch.float64) or cos_out.dtype != rho_out.dtype:
            raise TypeError("output coordinates must both be float32 or both float64")
        for t, n in ((rho_out, "RHO_OUT"), (cos_out, "COSALPHA_OUT")):
            if not t.is_cuda or not t.is_contiguous():
                raise TypeError(f"{n} must be a contiguous CUDA tensor")
        cd = _lib.COORD_F32 if rho_out.dtype == torch.float32 else _lib.COORD_F64
        check(self._lib.nfft2d_knab_set_points(self._h, rho_out.shape[0], rho_out.shape[1], _ptr(rho_out),
                                               _ptr(cos_out), cd), "nfft2d_knab_set_points")
        self.shape = tuple(rho_out.shape)
        self._keep = (rho_out, cos_out)

    def __call__(self, data: torch.Tensor, extrap=0.0, out: torch.Tensor | None = None) -> torch.Tensor:
        """Regrid INPUT_DATA (Nrows x Ncols complex CUDA tensor)."""
        if self.shape is None:
            raise RuntimeError("set_points first")
        if not data.is_cuda or data.dtype != self.cdtype or not data.is_contiguous():
            raise TypeError(f"INPUT_DATA must be a contiguous CUDA {self.cdtype} tensor")
        if tuple(data.shape) != (self.Nrows, self.Ncols):
            raise ValueError(f"INPUT_DATA must be {self.Nrows} x {self.Ncols}")
        if out is None:
            out = torch.empty(self.shape, dtype=self.cdtype, device=data.device)
        elif tuple(out.shape) != self.shape or out.dtype != self.cdtype or not out.is_contiguous():
            raise ValueError("out has the wrong shape or dtype")
        ev = complex(extrap)
        check(self._lib.nfft2d_knab_execute(self._h, ev.real, ev.imag, _ptr(data), _ptr(out)),
              "nfft2d_knab_execute")
        return out

    def synchronize(self) -> None:
        check(self._lib.nfft2d_knab_synchronize(self._h), "nfft2d_knab_synchronize")

    def info(self) -> dict:
        i = _lib.KnabInfo()
        check(self._lib.nfft2d_knab_get_info(self._h, ctypes.byref(i)), "nfft2d_knab_get_info")
        return i.as_dict()

    def plan_handle(self) -> ctypes.c_void_p:
        return ctypes.c_void_p(self._lib.nfft2d_knab_plan(self._h))


def knabNFFT2D(ExtrapVal, RHO_IN, COSALPHA_IN, INPUT_DATA: torch.Tensor, RHO_OUT: torch.Tensor,
               COSALPHA_OUT: torch.Tensor, B1: float, B2: float) -> torch.Tensor:
    """knabNFFT2D.m:1-79 on the GPU.  INPUT_DATA: Nrows x Ncols complex CUDA
    tensor (complex64 or complex128, which sets the precision); RHO_OUT,
    COSALPHA_OUT: len1 x len2 CUDA tensors; RHO_IN, COSALPHA_IN: vectors or
    meshgrid matrices (host or device)."""
    if not isinstance(INPUT_DATA, torch.Tensor) or INPUT_DATA.dtype not in (torch.complex64, torch.complex128):
        raise TypeError("INPUT_DATA must be a complex64 or complex128 CUDA tensor")
    precision = "f32" if INPUT_DATA.dtype == torch.complex64 else "f64"
    with Regridder(RHO_IN, COSALPHA_IN, B1, B2, precision=precision) as r:
        r.set_points(RHO_OUT.contiguous(), COSALPHA_OUT.contiguous())
        out = r(INPUT_DATA.contiguous(), ExtrapVal)
        r.synchronize()
    return out
