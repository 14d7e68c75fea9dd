"""Host-side mirror of the reference's 2D NFFT call surface, over the C ABI.

Device memory and streams come from PyTorch; every transform runs in
libnfft2d_gb300.so (hand-written sm_103a kernels + cuFFT).  There is no
CPU path: calls fail loudly if the library or a GPU is missing.

Reference interface mirrored (same names, argument meaning and layout):
  * ``NFFT2_2D(data, x1, x2, M1, M2)``   NFFT/NFFT2/Matlab/NFFT2_2D.m:1
  * ``NFFT1_2D(data, x1, x2)``           BP_FBP_FFBP/NFFT1_2D.m:1
  * ``NDFT2_2D(data, x, y, N, M)``        NFFT/NFFT2/Matlab/NDFT2_2D.m:1
  * ``NFFT2_2D_GPU(result, data, x, y, N1, N2, M)``  NFFT/NFFT2_2D.cu:329,413
  * ``NDFT2_2D_GPU(X, Y, u, v, d_in, d_out, Nu, Nv, M, N)``  NFFT/NDFT2_2D.cu:37
  * ``Calculate_cuFFT_plan_C2C_NFFT2_2D`` / ``..._Z2Z_...`` /
    ``Destroy_cuFFT_plan_NFFT2_2D``      NFFT/NFFT2_2D.cu:49-55
Coordinates of these functions are in the reference's grid units (a point
spans one period over [-N/2, N/2)); the window is fixed at c = 2, K = 6 as
in the reference.  ``Plan`` exposes the general interface (any sigma, K,
units, both signs, gradients, timing).
"""
from __future__ import annotations

import ctypes
import threading

import torch

from . import _lib
from ._lib import NFFT2DError, check

_REF_SIGMA = 2.0  # NFFT2_2D.cu:20 (cc), NFFT1_2D.m:9 (c)
_REF_K = 6        # NFFT2_2D.cu:21 (K),  NFFT1_2D.m:10 (K)


def _ptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    if t is None:
        return ctypes.c_void_p(0)
    return ctypes.c_void_p(t.data_ptr())


def _require_cuda(t: torch.Tensor, name: str, dtype: torch.dtype, numel: int | None = None) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must have dtype {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if numel is not None and t.numel() != numel:
        raise ValueError(f"{name} must have {numel} elements, got {t.numel()}")
    return t


class Plan:
    """A 2D NFFT plan: N1 x N2 coefficients, oversampling sigma, window
    half-width K (2K+1 taps per dimension), precision 'f32' or 'f64'.

    Wraps nfft2d_plan_create / set_points / forward / adjoint / spread_ref /
    type1 / type2 / grad_x.  The plan runs on a CUDA stream (default: torch's
    current stream at creation)."""

    def __init__(self, N1: int, N2: int, sigma: float = 2.0, K: int = 6, precision: str = "f32",
                 stream: torch.cuda.Stream | None = None):
        self._lib = _lib.load()
        if precision not in ("f32", "f64"):
            raise ValueError("precision must be 'f32' or 'f64'")
        self.N1, self.N2, self.sigma, self.K = int(N1), int(N2), float(sigma), int(K)
        self.precision = precision
        self.cdtype = torch.complex64 if precision == "f32" else torch.complex128
        self.rdtype = torch.float32 if precision == "f32" else torch.float64
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        h = ctypes.c_void_p()
        prec = _lib.F32 if precision == "f32" else _lib.F64
        check(self._lib.nfft2d_plan_create(ctypes.byref(h), self.N1, self.N2, self.sigma, self.K, prec,
                                           ctypes.c_void_p(self.stream.cuda_stream)), "nfft2d_plan_create")
        self._h = h
        self.M = 0
        self._keep = ()

    # -- life cycle -------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.nfft2d_plan_destroy(self._h)
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

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def set_stream(self, stream: torch.cuda.Stream) -> None:
        self.stream = stream
        check(self._lib.nfft2d_set_stream(self._h, ctypes.c_void_p(stream.cuda_stream)), "nfft2d_set_stream")

    def set_tuning(self, tile: int = -1, chunk: int = -1, gather_variant: int = -1, spread_variant: int = -1,
                   compensated: int = -1, fft_mode: int = -1, io_order: str | None = None) -> None:
        """Every argument left out keeps the plan's current setting.
        gather_variant / spread_variant: _lib.VARIANT_AUTO, _TILED or _DIRECT.
        fft_mode: -1 keep, 0 cuFFT 2D plan, 1 cuFFT row/band-column passes,
        2 hand-written passes fused with pad/fill/fold/crop (FP32, power-of-two
        grids; the default below 2048 x 2048 oversampled cells).
        io_order: None keep, 'caller' or 'binned' (per-point arrays in the
        plan's binned order, see permutation())."""
        io = -1 if io_order is None else {"caller": _lib.ORDER_CALLER, "binned": _lib.ORDER_BINNED}[io_order]
        t = _lib.Tuning(tile, chunk, gather_variant, spread_variant, compensated, fft_mode, io)
        check(self._lib.nfft2d_set_tuning(self._h, ctypes.byref(t)), "nfft2d_set_tuning")

    def permutation(self) -> torch.Tensor:
        """perm[i] = the caller's index of the point at binned position i (int32,
        on the device): with io_order 'binned', f_binned = f_caller[perm]."""
        perm = torch.empty(self.M, dtype=torch.int32, device=torch.device("cuda", torch.cuda.current_device()))
        check(self._lib.nfft2d_get_permutation(self._h, _ptr(perm)), "nfft2d_get_permutation")
        return perm

    def info(self) -> dict:
        i = _lib.Info()
        check(self._lib.nfft2d_get_info(self._h, ctypes.byref(i)), "nfft2d_get_info")
        return i.as_dict()

    def enable_timing(self, on: bool = True) -> None:
        check(self._lib.nfft2d_enable_timing(self._h, int(bool(on))), "nfft2d_enable_timing")

    def timings(self) -> dict:
        t = _lib.Timings()
        check(self._lib.nfft2d_get_timings(self._h, ctypes.byref(t)), "nfft2d_get_timings")
        return t.as_dict()

    def synchronize(self) -> None:
        check(self._lib.nfft2d_synchronize(self._h), "nfft2d_synchronize")

    # -- points -------------------------------------------------------------
    def set_points(self, x1: torch.Tensor, x2: torch.Tensor, units: str = "unit", sync: bool = True) -> None:
        """Bin and sort the points.  x1 pairs with N1 (rows), x2 with N2.
        units: 'grid' (reference: period N), 'unit' (period 1) or 'radians'.
        sync=False returns once the binning is enqueued: the transforms that
        follow on the plan's stream use the device-side result, and a
        non-finite coordinate is reported by the next synchronize()."""
        if x1.shape != x2.shape or x1.dim() != 1:
            raise ValueError("x1 and x2 must be 1-D tensors of equal length")
        if x1.dtype not in (torch.float32, torch.float64) or x2.dtype != x1.dtype:
            raise TypeError("coordinates must both be float32 or both float64")
        for t, name in ((x1, "x1"), (x2, "x2")):
            if t.is_cuda:
                _require_cuda(t, name, x1.dtype)
            elif not (t.is_pinned() and t.is_contiguous()):
                # page-locked host coordinates are read by the binning pass
                # over the host link, with no separate upload
                raise TypeError(f"{name} must be a CUDA tensor or a contiguous pinned CPU tensor")
        cd = _lib.COORD_F32 if x1.dtype == torch.float32 else _lib.COORD_F64
        M = x1.numel()
        fn = self._lib.nfft2d_set_points if sync else self._lib.nfft2d_set_points_async
        check(fn(self._h, M, _ptr(x1), _ptr(x2), cd, _lib.UNITS[units]), "nfft2d_set_points")
        self.M = M
        self._keep = (x1, x2)

    def bin_and_forward(self, x1: torch.Tensor, x2: torch.Tensor, F: torch.Tensor, units: str = "unit",
                        out: torch.Tensor | None = None, inputs_read: torch.cuda.Event | None = None) -> torch.Tensor:
        """set_points(x1, x2, sync=False) then forward(F), with the forward's
        padding and FFT running while the points are binned (they read only
        F).  x1, x2 and F may be CUDA tensors or contiguous pinned CPU
        tensors; a pinned F is uploaded after the coordinates have been read,
        while the rest of the binning runs.  inputs_read, a torch.cuda.Event,
        is recorded once the inputs have been read (the coordinates, and a
        pinned F): their buffers and the host link are free from there."""
        if x1.shape != x2.shape or x1.dim() != 1:
            raise ValueError("x1 and x2 must be 1-D tensors of equal length")
        if x1.dtype not in (torch.float32, torch.float64) or x2.dtype != x1.dtype:
            raise TypeError("coordinates must both be float32 or both float64")
        for t, name in ((x1, "x1"), (x2, "x2")):
            if t.is_cuda:
                _require_cuda(t, name, x1.dtype)
            elif not (t.is_pinned() and t.is_contiguous()):
                raise TypeError(f"{name} must be a CUDA tensor or a contiguous pinned CPU tensor")
        if F.is_cuda:
            F = self._coef(F)
            dev = F.device
        else:
            if not (F.is_pinned() and F.is_contiguous()):
                raise TypeError("F must be a CUDA tensor or a contiguous pinned CPU tensor")
            if F.dtype != self.cdtype or F.numel() != self.N1 * self.N2:
                raise ValueError(f"F must hold {self.N1 * self.N2} elements of {self.cdtype}")
            dev = x1.device if x1.is_cuda else torch.device("cuda", torch.cuda.current_device())
        M = x1.numel()
        out = torch.empty(M, dtype=self.cdtype, device=dev) if out is None else _require_cuda(
            out, "out", self.cdtype, M)
        ev = None
        if inputs_read is not None:
            inputs_read.record(self.stream)  # creates the event; the library records it again at the right point
            ev = ctypes.c_void_p(inputs_read.cuda_event)
        cd = _lib.COORD_F32 if x1.dtype == torch.float32 else _lib.COORD_F64
        check(self._lib.nfft2d_bin_and_forward(self._h, M, _ptr(x1), _ptr(x2), cd, _lib.UNITS[units], _ptr(F),
                                               _ptr(out), ev), "nfft2d_bin_and_forward")
        self.M = M
        self._keep = (x1, x2)
        return out

    # -- transforms ---------------------------------------------------------
    def _coef(self, F: torch.Tensor, name: str = "F") -> torch.Tensor:
        F = _require_cuda(F, name, self.cdtype, self.N1 * self.N2)
        return F

    def _vals(self, f: torch.Tensor, name: str = "f") -> torch.Tensor:
        return _require_cuda(f, name, self.cdtype, self.M)

    def type2(self, sign: int, F: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """f_p = sum_k F_k exp(sign 2 pi i k.x_p / N)."""
        F = self._coef(F)
        out = torch.empty(self.M, dtype=self.cdtype, device=F.device) if out is None else self._vals(out, "out")
        check(self._lib.nfft2d_type2(self._h, int(sign), _ptr(F), _ptr(out)), "nfft2d_type2")
        return out

    def type1(self, sign: int, f: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """F_k = sum_p f_p exp(sign 2 pi i k.x_p / N), returned N1 x N2."""
        f = self._vals(f)
        out = (torch.empty(self.N1, self.N2, dtype=self.cdtype, device=f.device) if out is None
               else self._coef(out, "out"))
        check(self._lib.nfft2d_type1(self._h, int(sign), _ptr(f), _ptr(out)), "nfft2d_type1")
        return out

    def forward(self, F: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """Type 2 with the reference's sign (NFFT1_2D)."""
        return self.type2(-1, F, out)

    def adjoint(self, f: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """Hermitian adjoint of forward: type 1 with sign +1."""
        return self.type1(+1, f, out)

    def spread_ref(self, f: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """Type 1 with the reference's sign (NFFT2_2D)."""
        return self.type1(-1, f, out)

    def grad_x(self, F: torch.Tensor, v: torch.Tensor, sign: int = -1):
        """(Re(conj(v) df/dx1), Re(conj(v) df/dx2)) for f = type2(sign, F),
        in the units given to set_points."""
        F = self._coef(F)
        v = self._vals(v, "v")
        g1 = torch.empty(self.M, dtype=self.rdtype, device=F.device)
        g2 = torch.empty_like(g1)
        check(self._lib.nfft2d_grad_x(self._h, int(sign), _ptr(F), _ptr(v), _ptr(g1), _ptr(g2)),
              "nfft2d_grad_x")
        return g1, g2


class Batch:
    """Many FP32 transforms of uneven size run together (nfft2d_batch_*):
    one batched cuFFT call per size group, one launch per stage for all
    transforms (the gather and spread once per window width), the whole
    stage sequence replayed as a CUDA graph.  K is one window half-width for
    all transforms or a sequence with one per transform."""

    def __init__(self, sizes, sigma: float = 2.0, K=6, stream: torch.cuda.Stream | None = None,
                 graph: bool = True):
        self._lib = _lib.load()
        self.sizes = [(int(a), int(b)) for a, b in sizes]
        self.count = len(self.sizes)
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        n1 = (ctypes.c_int * self.count)(*[a for a, _ in self.sizes])
        n2 = (ctypes.c_int * self.count)(*[b for _, b in self.sizes])
        h = ctypes.c_void_p()
        if isinstance(K, int):
            check(self._lib.nfft2d_batch_create(ctypes.byref(h), self.count, n1, n2, float(sigma), int(K),
                                                ctypes.c_void_p(self.stream.cuda_stream)), "nfft2d_batch_create")
        else:
            if len(K) != self.count:
                raise ValueError("K must be an int or hold one value per transform")
            ks = (ctypes.c_int * self.count)(*[int(k) for k in K])
            check(self._lib.nfft2d_batch_create_k(ctypes.byref(h), self.count, n1, n2, ks, float(sigma),
                                                  ctypes.c_void_p(self.stream.cuda_stream)), "nfft2d_batch_create_k")
        self._h = h
        self.M = [0] * self.count
        self._keep = ()
        if not graph:
            check(self._lib.nfft2d_batch_set_graph(self._h, 0), "nfft2d_batch_set_graph")

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.nfft2d_batch_destroy(self._h)
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

    @staticmethod
    def _ptrs(ts):
        return (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])

    def set_points(self, x1s, x2s, units: str = "unit") -> None:
        if len(x1s) != self.count or len(x2s) != self.count:
            raise ValueError("one coordinate pair per transform")
        dt = x1s[0].dtype
        for a, b in zip(x1s, x2s):
            _require_cuda(a, "x1", dt)
            _require_cuda(b, "x2", dt)
            if a.shape != b.shape:
                raise ValueError("x1 and x2 must match")
        M = (ctypes.c_longlong * self.count)(*[a.numel() for a in x1s])
        cd = _lib.COORD_F32 if dt == torch.float32 else _lib.COORD_F64
        check(self._lib.nfft2d_batch_set_points(self._h, M, self._ptrs(x1s), self._ptrs(x2s), cd, _lib.UNITS[units]),
              "nfft2d_batch_set_points")
        self.M = [a.numel() for a in x1s]
        self._keep = (list(x1s), list(x2s))

    def forward(self, Fs, outs=None):
        for (n1, n2), F in zip(self.sizes, Fs):
            _require_cuda(F, "F", torch.complex64, n1 * n2)
        if outs is None:
            outs = [torch.empty(m, dtype=torch.complex64, device=Fs[0].device) for m in self.M]
        check(self._lib.nfft2d_batch_forward(self._h, self._ptrs(Fs), self._ptrs(outs)), "nfft2d_batch_forward")
        return outs

    def adjoint(self, fs, outs=None):
        for m, f in zip(self.M, fs):
            _require_cuda(f, "f", torch.complex64, m)
        if outs is None:
            outs = [torch.empty(n1 * n2, dtype=torch.complex64, device=fs[0].device) for n1, n2 in self.sizes]
        check(self._lib.nfft2d_batch_adjoint(self._h, self._ptrs(fs), self._ptrs(outs)), "nfft2d_batch_adjoint")
        return outs

    def spread_ref(self, fs, outs=None):
        """Type 1 with the reference's sign (NFFT2_2D_GPU) for every transform."""
        for m, f in zip(self.M, fs):
            _require_cuda(f, "f", torch.complex64, m)
        if outs is None:
            outs = [torch.empty(n1 * n2, dtype=torch.complex64, device=fs[0].device) for n1, n2 in self.sizes]
        check(self._lib.nfft2d_batch_spread_ref(self._h, self._ptrs(fs), self._ptrs(outs)), "nfft2d_batch_spread_ref")
        return outs

    def far_field(self, X, Y, excitations, scale_x: float, scale_y: float, filter: torch.Tensor | None = None,
                  outs=None):
        """The PSO far-field step for every particle (nfft2d_batch_far_field,
        Synthesis/PSO/Synthesis.cu:385-405): element positions X[t], Y[t]
        (float32, one tensor per particle, equal lengths), excitations[t]
        (complex64), the FP32 scales of :388-389 (see pso_far_field_scales)
        and the spectral filter (float32, N1*N2).  Returns the far fields."""
        if len(X) != self.count or len(Y) != self.count or len(excitations) != self.count:
            raise ValueError("one X, Y and excitation per transform")
        M = X[0].numel()
        for a, b, e in zip(X, Y, excitations):
            _require_cuda(a, "X", torch.float32, M)
            _require_cuda(b, "Y", torch.float32, M)
            _require_cuda(e, "excitations", torch.complex64, M)
        if filter is not None:
            n1, n2 = self.sizes[0]
            _require_cuda(filter, "filter", torch.float32, n1 * n2)
        if outs is None:
            outs = [torch.empty(n1 * n2, dtype=torch.complex64, device=X[0].device) for n1, n2 in self.sizes]
        check(self._lib.nfft2d_batch_far_field(self._h, M, self._ptrs(X), self._ptrs(Y), float(scale_x),
                                               float(scale_y), self._ptrs(excitations),
                                               _ptr(filter), self._ptrs(outs)), "nfft2d_batch_far_field")
        self.M = [M] * self.count
        self._keep = (list(X), list(Y))
        return outs

    def synchronize(self) -> None:
        check(self._lib.nfft2d_batch_synchronize(self._h), "nfft2d_batch_synchronize")


def pso_spectral_grid(u_max: float, v_max: float, a_prime: float, b_prime: float):
    """Nu, Nv of the PSO synthesis' spectral grid (Synthesis/PSO/Synthesis.cu:82-83):
    Nu = (int)(u_max / (pi / a')) + 1; the far field is 2 Nv x 2 Nu."""
    import math
    return int(u_max / (math.pi / a_prime)) + 1, int(v_max / (math.pi / b_prime)) + 1


def pso_far_field_scales(Nu: int, Nv: int, a_prime_f: float, b_prime_f: float):
    """The FP32 coordinate scales of Synthesis.cu:388-389,
    float(2 Nu (pi / a')) / (float(2) pi), rounded to FP32 as the reference
    passes them to vectorMulConstant<float>."""
    import math

    import numpy as np
    f32 = np.float32
    sx = float(f32(2 * Nu * (math.pi / float(f32(a_prime_f))))) / (2.0 * math.pi)
    sy = float(f32(2 * Nv * (math.pi / float(f32(b_prime_f))))) / (2.0 * math.pi)
    return float(f32(sx)), float(f32(sy))


# ---------------------------------------------------------------------------
# Reference call surface (c = 2, K = 6, grid-unit coordinates)
# ---------------------------------------------------------------------------
_cache_lock = threading.Lock()
_plan_cache: dict[tuple, Plan] = {}


def _cached_plan(N1: int, N2: int, precision: str) -> Plan:
    key = (int(N1), int(N2), precision, torch.cuda.current_device())
    with _cache_lock:
        p = _plan_cache.get(key)
        if p is None:
            p = Plan(N1, N2, _REF_SIGMA, _REF_K, precision)
            _plan_cache[key] = p
        return p


def _prec_of(t: torch.Tensor) -> str:
    if t.dtype in (torch.complex64, torch.float32):
        return "f32"
    if t.dtype in (torch.complex128, torch.float64):
        return "f64"
    raise TypeError(f"unsupported dtype {t.dtype}")


def Calculate_cuFFT_plan_C2C_NFFT2_2D(N1: int, N2: int) -> None:
    """NFFT2_2D.cu:49: create the single-precision plan for N1 x N2 outputs."""
    _cached_plan(N1, N2, "f32")


def Calculate_cuFFT_plan_Z2Z_NFFT2_2D(N1: int, N2: int) -> None:
    """NFFT2_2D.cu:50: create the double-precision plan for N1 x N2 outputs."""
    _cached_plan(N1, N2, "f64")


def Destroy_cuFFT_plan_NFFT2_2D() -> None:
    """NFFT2_2D.cu:55: release every cached plan."""
    with _cache_lock:
        for p in _plan_cache.values():
            p.close()
        _plan_cache.clear()


def NFFT2_2D_GPU(result: torch.Tensor, data: torch.Tensor, x: torch.Tensor, y: torch.Tensor,
                 N1: int, N2: int, M: int) -> None:
    """NFFT2_2D.cu:329/413: result[i, j] = sum_p data[p] exp(-2 pi i ((i-N1/2) x_p/N1 + (j-N2/2) y_p/N2)),
    x, y in grid units; result is N1*N2 complex (row-major), written in place."""
    prec = _prec_of(data)
    p = _cached_plan(N1, N2, prec)
    if x.numel() < M or y.numel() < M or data.numel() < M:
        raise ValueError("x, y and data must hold at least M entries")
    p.set_points(x[:M], y[:M], units="grid")
    p.spread_ref(data[:M], out=result.view(-1) if result.dim() != 1 else result)
    p.synchronize()


def NDFT2_2D_GPU(X: torch.Tensor, Y: torch.Tensor, u: torch.Tensor, v: torch.Tensor, d_in: torch.Tensor,
                 d_out: torch.Tensor, Nu: int, Nv: int, M: int, N: int, sign: int = -1) -> None:
    """NDFT2_2D.cu:37-72: d_out[q] = sum_p d_in[p] exp(-2 pi i (u_q X_p/Nu + v_q Y_p/Nv)), FP64,
    matrix-free (no cuBLAS handle, no file dump)."""
    for t, n in ((X, "X"), (Y, "Y"), (u, "u"), (v, "v")):
        _require_cuda(t, n, torch.float64)
    _require_cuda(d_in, "d_in", torch.complex128)
    _require_cuda(d_out, "d_out", torch.complex128)
    lib = _lib.load()
    check(lib.nfft2d_ndft2d_f64(_ptr(X), _ptr(Y), _ptr(u), _ptr(v), _ptr(d_in), _ptr(d_out), int(Nu), int(Nv),
                                int(M), int(N), int(sign), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
          "nfft2d_ndft2d_f64")


def NFFT2_2D(data: torch.Tensor, x1: torch.Tensor, x2: torch.Tensor, M1: int, M2: int) -> torch.Tensor:
    """NFFT2_2D.m:1: transf(k1, k2) = sum_p data_p exp(-2 pi i (k1 x1_p / M1 + k2 x2_p / M2)),
    k in [-M/2, M/2), returned M1 x M2 (row <-> x1)."""
    p = _cached_plan(M1, M2, _prec_of(data))
    p.set_points(x1.contiguous(), x2.contiguous(), units="grid")
    return p.spread_ref(data.contiguous().view(-1))


def NFFT1_2D(data: torch.Tensor, x1: torch.Tensor, x2: torch.Tensor) -> torch.Tensor:
    """BP_FBP_FFBP/NFFT1_2D.m:1: result_p = sum_k data(k1, k2) exp(-2 pi i (k1 x1_p / N1 + k2 x2_p / N2)),
    data N1 x N2 with row <-> k1 = i - N1/2."""
    N1, N2 = data.shape
    p = _cached_plan(N1, N2, _prec_of(data))
    p.set_points(x1.contiguous(), x2.contiguous(), units="grid")
    return p.forward(data.contiguous())


def NDFT2_2D(data: torch.Tensor, x: torch.Tensor, y: torch.Tensor, N: int, M: int) -> torch.Tensor:
    """NDFT2_2D.m:1 layout: returns N x M with element (r, s) pairing the
    y-frequency v = r - M/2 ... as in the MATLAB reshape: (r, s) holds
    sum_p data_p exp(-2 pi i (x_p u_s / N + y_p v_r / M)), u_s = s - N/2,
    v_r = r - M/2, for N == M (the MATLAB divides the y-term by N, which is
    the same thing when N == M; for N != M the intended /M is used).  Exact
    FP64 direct sum on the GPU."""
    if N != M:
        raise NFFT2DError(_lib.ERR_UNSUPPORTED, "NDFT2_2D: the reference layout is defined for N == M")
    dev = data.device
    u = torch.arange(N, device=dev, dtype=torch.float64) - N // 2
    v = torch.arange(M, device=dev, dtype=torch.float64) - M // 2
    # output (r, s) row-major: q = r * M + s; r <-> v, s <-> u
    vv, uu = torch.meshgrid(v, u, indexing="ij")
    out = torch.empty(N * M, dtype=torch.complex128, device=dev)
    NDFT2_2D_GPU(x.to(torch.float64).contiguous(), y.to(torch.float64).contiguous(), uu.reshape(-1).contiguous(),
                 vv.reshape(-1).contiguous(), data.to(torch.complex128).contiguous(), out, N, M, x.numel(), N * M)
    return out.view(N, M)


__all__ = ["Plan", "Batch", "NFFT2DError", "NFFT2_2D", "NFFT1_2D", "NDFT2_2D", "NFFT2_2D_GPU", "NDFT2_2D_GPU",
           "Calculate_cuFFT_plan_C2C_NFFT2_2D", "Calculate_cuFFT_plan_Z2Z_NFFT2_2D", "Destroy_cuFFT_plan_NFFT2_2D"]
