"""ctypes binding of libnfft2d_gb300.so (the C ABI declared in
include/nfft2d_gb300.h).

The library is built in-tree (``miscellaneous_gb300/lib``) by
``miscellaneous_gb300.build.build()``.  Loading fails loudly when it is
missing: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes
import os
import re

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libnfft2d_gb300.so")
HEADER_PATH = os.path.join(os.path.dirname(_PKG), "include", "nfft2d_gb300.h")

# status codes (nfft2d_gb300.h)
OK = 0
ERR_INVALID_ARG = -1
ERR_OOM = -2
ERR_CUDA = -3
ERR_CUFFT = -4
ERR_NO_POINTS = -5
ERR_NONFINITE = -6
ERR_DEVICE_TIMEOUT = -7
ERR_DEVICE_BOUNDS = -8
ERR_UNSUPPORTED = -9
ERR_INTERNAL = -10
ERR_SCRATCH_LIMIT = -11

F32 = 0
F64 = 1
COORD_F32 = 0
COORD_F64 = 1
UNITS = {"grid": 0, "unit": 1, "radians": 2}
VARIANT_AUTO, VARIANT_TILED, VARIANT_DIRECT = 0, 1, 2


class Info(ctypes.Structure):
    _fields_ = [
        ("N1", ctypes.c_int), ("N2", ctypes.c_int), ("sigma", ctypes.c_double), ("K", ctypes.c_int),
        ("precision", ctypes.c_int), ("n1", ctypes.c_int), ("n2", ctypes.c_int), ("halo", ctypes.c_int),
        ("rows", ctypes.c_int), ("cols", ctypes.c_int), ("tile", ctypes.c_int), ("tiles1", ctypes.c_int),
        ("tiles2", ctypes.c_int), ("patch_rows", ctypes.c_int), ("patch_cols", ctypes.c_int),
        ("chunk", ctypes.c_int), ("gather_variant", ctypes.c_int), ("spread_variant", ctypes.c_int),
        ("M", ctypes.c_longlong), ("n_chunks", ctypes.c_longlong), ("workspace_bytes", ctypes.c_size_t),
        ("fft_mode", ctypes.c_int),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


ORDER_CALLER = 0
ORDER_BINNED = 1


class Tuning(ctypes.Structure):
    _fields_ = [("tile", ctypes.c_int), ("chunk", ctypes.c_int), ("gather_variant", ctypes.c_int),
                ("spread_variant", ctypes.c_int), ("compensated", ctypes.c_int), ("fft_mode", ctypes.c_int),
                ("io_order", ctypes.c_int)]


class Timings(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in
                ("sort_ms", "pad_ms", "fft_type2_ms", "halo_fill_ms", "gather_ms", "spread_ms", "fold_ms",
                 "fft_type1_ms", "crop_ms")]

    def as_dict(self) -> dict:
        return {name: float(getattr(self, name)) for name, _ in self._fields_}


class KnabInfo(ctypes.Structure):
    _fields_ = [("Nrows", ctypes.c_int), ("Ncols", ctypes.c_int), ("kgn", ctypes.c_int), ("kgm", ctypes.c_int),
                ("T1", ctypes.c_double), ("T2", ctypes.c_double), ("a", ctypes.c_int), ("b", ctypes.c_int),
                ("N1", ctypes.c_int), ("N2", ctypes.c_int), ("len1", ctypes.c_int), ("len2", ctypes.c_int),
                ("masked_lines", ctypes.c_int)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class NFFT2DError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = status_string(status) if _lib is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


class Sar(ctypes.Structure):
    """nfft2d_sar: propagation speed, centre frequency, bandwidth, maximum frequency."""
    _fields_ = [("c", ctypes.c_double), ("fc", ctypes.c_double), ("bw", ctypes.c_double), ("f_max", ctypes.c_double)]


class FfbpStats(ctypes.Structure):
    _fields_ = [("depth", ctypes.c_int), ("regrids", ctypes.c_int), ("leaves", ctypes.c_int),
                ("leaf_points", ctypes.c_longlong), ("regrid_points", ctypes.c_longlong),
                ("raster_cells", ctypes.c_longlong)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None

_P = ctypes.c_void_p
_I = ctypes.c_int
_LL = ctypes.c_longlong
_D = ctypes.c_double

_SIGNATURES = {
    "nfft2d_plan_create": (_I, [ctypes.POINTER(_P), _I, _I, _D, _I, _I, _P]),
    "nfft2d_plan_destroy": (_I, [_P]),
    "nfft2d_set_stream": (_I, [_P, _P]),
    "nfft2d_set_tuning": (_I, [_P, ctypes.POINTER(Tuning)]),
    "nfft2d_get_info": (_I, [_P, ctypes.POINTER(Info)]),
    "nfft2d_get_permutation": (_I, [_P, _P]),
    "nfft2d_layout_query": (_I, [_I, _I, _D, _I, _I, _I, ctypes.POINTER(Info)]),
    "nfft2d_set_points": (_I, [_P, _LL, _P, _P, _I, _I]),
    "nfft2d_set_points_async": (_I, [_P, _LL, _P, _P, _I, _I]),
    "nfft2d_bin_and_forward": (_I, [_P, _LL, _P, _P, _I, _I, _P, _P, _P]),
    "nfft2d_forward": (_I, [_P, _P, _P]),
    "nfft2d_adjoint": (_I, [_P, _P, _P]),
    "nfft2d_spread_ref": (_I, [_P, _P, _P]),
    "nfft2d_type2": (_I, [_P, _I, _P, _P]),
    "nfft2d_type1": (_I, [_P, _I, _P, _P]),
    "nfft2d_grad_x": (_I, [_P, _I, _P, _P, _P, _P]),
    "nfft2d_synchronize": (_I, [_P]),
    "nfft2d_enable_timing": (_I, [_P, _I]),
    "nfft2d_get_timings": (_I, [_P, ctypes.POINTER(Timings)]),
    "nfft2d_status_string": (ctypes.c_char_p, [_I]),
    "nfft2d_device_count": (_I, []),
    "nfft2d_selftest_wait_timeout": (_I, [_I, _P]),
    "nfft2d_plan_selftest_wait_timeout": (_I, [_P, _I]),
    "nfft2d_ndft2d_f64": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _LL, _LL, _I, _P]),
    "nfft2d_forward_small_noalloc": (_I, [_I, _I, _I, _LL, _P, _P, _I, _P, _P, _P]),
    "nfft2d_batch_create": (_I, [ctypes.POINTER(_P), _I, _P, _P, _D, _I, _P]),
    "nfft2d_batch_create_k": (_I, [ctypes.POINTER(_P), _I, _P, _P, _P, _D, _P]),
    "nfft2d_batch_destroy": (_I, [_P]),
    "nfft2d_batch_set_points": (_I, [_P, _P, _P, _P, _I, _I]),
    "nfft2d_batch_forward": (_I, [_P, _P, _P]),
    "nfft2d_batch_adjoint": (_I, [_P, _P, _P]),
    "nfft2d_batch_spread_ref": (_I, [_P, _P, _P]),
    "nfft2d_batch_set_graph": (_I, [_P, _I]),
    "nfft2d_batch_far_field": (_I, [_P, _LL, _P, _P, ctypes.c_float, ctypes.c_float, _P, _P, _P]),
    "nfft2d_batch_synchronize": (_I, [_P]),
    "nfft2d_batch_selftest_wait_timeout": (_I, [_P, _I]),
    "nfft2d_knab_window": (_I, [_D, _D, _I, _I, _P, _I, ctypes.POINTER(_I)]),
    "nfft2d_knab_create": (_I, [ctypes.POINTER(_P), _I, _I, _P, _P, _D, _D, _I, _P]),
    "nfft2d_knab_destroy": (_I, [_P]),
    "nfft2d_knab_set_points": (_I, [_P, _I, _I, _P, _P, _I]),
    "nfft2d_knab_execute": (_I, [_P, _D, _D, _P, _P]),
    "nfft2d_knab_get_info": (_I, [_P, ctypes.POINTER(KnabInfo)]),
    "nfft2d_knab_synchronize": (_I, [_P]),
    "nfft2d_knab_plan": (_P, [_P]),
    "nfft2d_knab_nfft2d": (_I, [_D, _D, _P, _I, _P, _I, _P, _P, _P, _I, _I, _D, _D, _I, _P, _P]),
    "nfft2d_nufft3_2d": (_I, [_P, _P, _P, _P, _P, _P, _D, _LL, _LL, _I, _P]),
    "nfft2d_ffbp_polar": (_I, [ctypes.POINTER(Sar), _I, _P, _P, _P, _P, _I, _P, _I, _I, _I, _I, _P, _P, _I, _P, _P,
                               ctypes.POINTER(FfbpStats)]),
}


def header_functions(path: str = HEADER_PATH) -> list[str]:
    """Names of every function declared in include/nfft2d_gb300.h."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nfft2d_[a-z0-9_]+)\s*\(", text)))


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: the CUDA extension has not been built "
            "(run `python -c 'import __graft_entry__ as g; g.build()'`). "
            "This package has no CPU fallback.")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(status: int) -> str:
    return load().nfft2d_status_string(int(status)).decode()


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise NFFT2DError(status, what)
