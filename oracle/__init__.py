"""CPU oracle for the 2D NFFT path -- TEST INFRASTRUCTURE ONLY.

This package is the checker, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline and reference
legs) import it.  ``miscellaneous_gb300`` never imports it and has no CPU
fallback.

It wraps ``nfft2d_oracle.c`` (an FP64 C restatement of the reference's
``BP_FBP_FFBP/NFFT1_2D.m``, ``NFFT/NFFT2/Matlab/NFFT2_2D.m``,
``NFFT/NFFT2/Matlab/NDFT2_2D.m`` and ``NFFT/NDFT2_2D.cu``, and of the
Knab-window regridding ``BP_FBP_FFBP/knabNFFT2D.m`` with
``NFFT_Based_Selvas_Approach_for_Signal_Interp_2D.m``, ``KnabWindow.m`` and
``ConvWindow.m``) through ctypes.
All coordinates here are in the reference's grid units (period N per
dimension); callers with coordinates in [-0.5, 0.5) multiply by N first.

Parity pinning: the reference ships no golden vectors and its MATLAB code
cannot run here, so the oracle is pinned by (1) the reference's own
acceptance test (Test_NFFT2_2D.m:24-29: NFFT vs the NDFT direct sum),
(2) fixtures from an independent numpy transliteration of the MATLAB files
(tests/golden/make_golden.py) and (3) analytic known answers.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "nfft2d_oracle.c")
_BUILD_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD_DIR, "liboracle_nfft2d.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the C restatement with gcc + OpenMP into oracle/_build/."""
    os.makedirs(_BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp",
           "-D_DEFAULT_SOURCE", _SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(_LIB_PATH)
    D = ctypes.c_double
    L = ctypes.c_long
    I = ctypes.c_int
    P = ctypes.c_void_p
    sig = {
        "oracle_version": (I, []),
        "oracle_set_threads": (None, [I]),
        "oracle_get_threads": (I, []),
        "oracle_bessel_i0": (D, [D]),
        "oracle_kb_alpha": (D, [D]),
        "oracle_phi_hat": (D, [D, I, D]),
        "oracle_phi_hat_deriv": (D, [D, I, D]),
        "oracle_phi": (D, [D, I, D]),
        "oracle_fft2d": (None, [P, L, L, I]),
        "oracle_nfft1_2d": (I, [P, L, L, P, P, L, D, I, I, P]),
        "oracle_nfft1_1d": (I, [P, L, P, L, D, I, I, P]),
        "oracle_ndft3_2d": (None, [P, P, P, L, P, P, L, P]),
        "oracle_nufft3_2d": (I, [P, P, P, L, P, P, L, D, D, P, P]),
        "oracle_nfft1_2d_grad": (I, [P, L, L, P, P, L, D, I, I, P, P]),
        "oracle_nfft2_2d": (I, [P, P, P, L, L, L, D, I, I, P]),
        "oracle_ndft_type2": (None, [P, L, L, P, P, L, I, P]),
        "oracle_ndft_type2_grad": (None, [P, L, L, P, P, L, I, P, P]),
        "oracle_ndft_type1": (None, [P, P, P, L, L, L, I, P]),
        "oracle_ndft2_2d_general": (None, [P, P, P, P, P, L, L, L, L, P]),
        "oracle_ndft2_2d_matlab": (None, [P, P, P, L, L, L, P]),
        "oracle_conv_window": (D, [D, D, D]),
        "oracle_conv_window_integral": (D, [D, D, D, D, D]),
        "oracle_knab_window": (L, [D, D, I, L, P]),
        "oracle_knab_nfft2d": (I, [D, D, P, L, P, L, P, P, P, L, L, D, D, I, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> None:
    _load().oracle_set_threads(int(n))


def get_threads() -> int:
    return int(_load().oracle_get_threads())


def bessel_i0(x: float) -> float:
    return _load().oracle_bessel_i0(float(x))


def kb_alpha(c: float) -> float:
    return _load().oracle_kb_alpha(float(c))


def phi_hat(t: float, K: int, alpha: float) -> float:
    return _load().oracle_phi_hat(float(t), int(K), float(alpha))


def phi_hat_deriv(t: float, K: int, alpha: float) -> float:
    return _load().oracle_phi_hat_deriv(float(t), int(K), float(alpha))


def phi(xi: float, K: int, alpha: float) -> float:
    return _load().oracle_phi(float(xi), int(K), float(alpha))


def fft2(a, sign: int = -1) -> np.ndarray:
    a = _c128(a).copy()
    _load().oracle_fft2d(_ptr(a), a.shape[0], a.shape[1], int(sign))
    return a


def nfft1_2d(F, x1, x2, c: float = 2.0, K: int = 6, sign: int = -1) -> np.ndarray:
    """Restated BP_FBP_FFBP/NFFT1_2D.m: forward type-2, grid-unit points."""
    F = _c128(F)
    x1, x2 = _f64(x1), _f64(x2)
    out = np.zeros(x1.shape[0], dtype=np.complex128)
    rc = _load().oracle_nfft1_2d(_ptr(F), F.shape[0], F.shape[1], _ptr(x1), _ptr(x2),
                                 x1.shape[0], float(c), int(K), int(sign), _ptr(out))
    if rc != 0:
        raise ValueError("oracle_nfft1_2d: invalid grid (N must be even, c*N an even integer)")
    return out


def nfft1_2d_grad(F, x1, x2, c: float = 2.0, K: int = 6, sign: int = -1):
    F = _c128(F)
    x1, x2 = _f64(x1), _f64(x2)
    g1 = np.zeros(x1.shape[0], dtype=np.complex128)
    g2 = np.zeros_like(g1)
    rc = _load().oracle_nfft1_2d_grad(_ptr(F), F.shape[0], F.shape[1], _ptr(x1), _ptr(x2),
                                      x1.shape[0], float(c), int(K), int(sign), _ptr(g1), _ptr(g2))
    if rc != 0:
        raise ValueError("oracle_nfft1_2d_grad: invalid grid")
    return g1, g2


def nfft2_2d(d, x1, x2, N1: int, N2: int, c: float = 2.0, K: int = 6, sign: int = -1) -> np.ndarray:
    """Restated NFFT/NFFT2/Matlab/NFFT2_2D.m: spreading type-1, grid-unit points."""
    d = _c128(d)
    x1, x2 = _f64(x1), _f64(x2)
    out = np.zeros((N1, N2), dtype=np.complex128)
    rc = _load().oracle_nfft2_2d(_ptr(d), _ptr(x1), _ptr(x2), x1.shape[0], int(N1), int(N2),
                                 float(c), int(K), int(sign), _ptr(out))
    if rc != 0:
        raise ValueError("oracle_nfft2_2d: invalid grid (N must be even, c*N an even integer)")
    return out


def ndft_type2(F, x1, x2, sign: int = -1) -> np.ndarray:
    """Exact f_p = sum_k F_k exp(sign 2 pi i k.x_p / N), grid-unit points."""
    F = _c128(F)
    x1, x2 = _f64(x1), _f64(x2)
    out = np.zeros(x1.shape[0], dtype=np.complex128)
    _load().oracle_ndft_type2(_ptr(F), F.shape[0], F.shape[1], _ptr(x1), _ptr(x2),
                              x1.shape[0], int(sign), _ptr(out))
    return out


def ndft_type2_grad(F, x1, x2, sign: int = -1):
    F = _c128(F)
    x1, x2 = _f64(x1), _f64(x2)
    g1 = np.zeros(x1.shape[0], dtype=np.complex128)
    g2 = np.zeros_like(g1)
    _load().oracle_ndft_type2_grad(_ptr(F), F.shape[0], F.shape[1], _ptr(x1), _ptr(x2),
                                   x1.shape[0], int(sign), _ptr(g1), _ptr(g2))
    return g1, g2


def ndft_type1(d, x1, x2, N1: int, N2: int, sign: int = -1) -> np.ndarray:
    """Exact F_k = sum_p d_p exp(sign 2 pi i k.x_p / N), grid-unit points."""
    d = _c128(d)
    x1, x2 = _f64(x1), _f64(x2)
    out = np.zeros((N1, N2), dtype=np.complex128)
    _load().oracle_ndft_type1(_ptr(d), _ptr(x1), _ptr(x2), x1.shape[0], int(N1), int(N2),
                              int(sign), _ptr(out))
    return out


def ndft2_2d_general(X, Y, u, v, d, Nu: int, Nv: int) -> np.ndarray:
    """NDFT2_2D_GPU semantics (NFFT/NDFT2_2D.cu:15-32,67) at arbitrary frequencies."""
    X, Y, u, v = _f64(X), _f64(Y), _f64(u), _f64(v)
    d = _c128(d)
    out = np.zeros(u.shape[0], dtype=np.complex128)
    _load().oracle_ndft2_2d_general(_ptr(X), _ptr(Y), _ptr(u), _ptr(v), _ptr(d), int(Nu), int(Nv),
                                    X.shape[0], u.shape[0], _ptr(out))
    return out


def ndft2_2d_matlab(data, x, y, N: int, M: int) -> np.ndarray:
    """Literal NDFT2_2D.m (layout and the /N of both phase terms kept)."""
    data = _c128(data)
    x, y = _f64(x), _f64(y)
    out = np.zeros((N, M), dtype=np.complex128)
    _load().oracle_ndft2_2d_matlab(_ptr(data), _ptr(x), _ptr(y), x.shape[0], int(N), int(M), _ptr(out))
    return out


def rel_l2(a, b) -> float:
    """sqrt(sum|a-b|^2 / sum|b|^2), the error measure of Test_NFFT2_2D.m:28."""
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    den = np.sqrt(np.sum(np.abs(b) ** 2))
    return float(np.sqrt(np.sum(np.abs(a - b) ** 2)) / den) if den > 0 else float(np.sqrt(np.sum(np.abs(a) ** 2)))


def nfft1_1d(data, x, c: float = 2.0, K: int = 6, sign: int = -1) -> np.ndarray:
    """Restated NFFT1_1D.m (BP_FBP_FFBP/NFFT1_1D.m:1-51): the 1D type-2 NFFT
    of N samples at points x in grid units (period N)."""
    data = _c128(data).ravel()
    x = _f64(x).ravel()
    out = np.zeros(x.size, dtype=np.complex128)
    rc = _load().oracle_nfft1_1d(_ptr(data), data.size, _ptr(x), x.size, float(c), int(K), int(sign), _ptr(out))
    if rc != 0:
        raise ValueError("oracle_nfft1_1d: N must be even and c*N an even integer")
    return out


def ndft3_2d(x, y, f, s, t) -> np.ndarray:
    """Exact type-3 sum F_k = sum_j f_j exp(-i (s_k x_j + t_k y_j)) (FP64)."""
    x, y, s, t = (_f64(v).ravel() for v in (x, y, s, t))
    f = _c128(f).ravel()
    out = np.zeros(s.size, dtype=np.complex128)
    _load().oracle_ndft3_2d(_ptr(x), _ptr(y), _ptr(f), x.size, _ptr(s), _ptr(t), s.size, _ptr(out))
    return out


def nufft3_2d(x, y, f, s, t, eps: float, R: float = 2.2):
    """Restated NUFFT_2D_CPU (NFFT/NFFT3/C/NFFT3_2D_C.cpp:199-312): Gaussian
    gridding type-3 NUFFT.  Returns (F, {"Mrx", "Mry", "msp"})."""
    x, y, s, t = (_f64(v).ravel() for v in (x, y, s, t))
    f = _c128(f).ravel()
    out = np.zeros(s.size, dtype=np.complex128)
    info = np.zeros(3, dtype=np.int64)
    rc = _load().oracle_nufft3_2d(_ptr(x), _ptr(y), _ptr(f), x.size, _ptr(s), _ptr(t), s.size, float(eps), float(R),
                                  _ptr(out), _ptr(info))
    if rc != 0:
        raise ValueError("oracle_nufft3_2d: degenerate input extent")
    return out, dict(Mrx=int(info[0]), Mry=int(info[1]), msp=int(info[2]))


def conv_window(f: float, B: float, T: float) -> float:
    """Restated ConvWindow.m: the approximate prolate window of Selva's method."""
    return _load().oracle_conv_window(float(f), float(B), float(T))


def knab_window(T: float, B: float, P: int, N: int):
    """Restated KnabWindow.m: returns (G, kg), G over frequencies -kg..kg."""
    lib = _load()
    kg = int(lib.oracle_knab_window(float(T), float(B), int(P), int(N), None))
    if kg < 0:
        return np.zeros(0), kg
    G = np.zeros(2 * kg + 1)
    lib.oracle_knab_window(float(T), float(B), int(P), int(N), _ptr(G))
    return G, kg


def knab_nfft2d(extrap, rho_in, cos_in, data, rho_out, cos_out, B1: float, B2: float, direct: bool = False):
    """Restated knabNFFT2D.m (with Selva's NFFT interpolation).

    rho_in: the Ncols input range samples (RHO_IN(1, :)); cos_in: the Nrows
    input angle samples (COSALPHA_IN(:, 1)); data: Nrows x Ncols; rho_out,
    cos_out: len1 x len2.  Returns (out len1 x len2, {"a", "b", "kgn", "kgm"}).
    direct=True evaluates the same trigonometric sum exactly instead of by
    NFFT1_2D."""
    rho_in, cos_in = _f64(rho_in).ravel(), _f64(cos_in).ravel()
    data = _c128(data)
    rho_out, cos_out = _f64(rho_out), _f64(cos_out)
    if rho_out.ndim != 2 or rho_out.shape != cos_out.shape:
        raise ValueError("rho_out and cos_out must be equal-shape 2-D arrays")
    Nrows, Ncols = data.shape
    if rho_in.size != Ncols or cos_in.size != Nrows:
        raise ValueError("axis lengths must match the data")
    len1, len2 = rho_out.shape
    out = np.zeros((len1, len2), dtype=np.complex128)
    info = np.zeros(4, dtype=np.int64)
    ev = complex(extrap)
    rc = _load().oracle_knab_nfft2d(ev.real, ev.imag, _ptr(rho_in), Ncols, _ptr(cos_in), Nrows, _ptr(data),
                                    _ptr(rho_out), _ptr(cos_out), len1, len2, float(B1), float(B2), int(bool(direct)),
                                    _ptr(out), _ptr(info))
    if rc != 0:
        raise ValueError("oracle_knab_nfft2d: configuration the reference cannot run")
    return out, dict(a=int(info[0]), b=int(info[1]), kgn=int(info[2]), kgm=int(info[3]))
