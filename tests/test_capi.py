"""C-ABI checks that need no GPU: the library loads, exports every function
declared in include/nfft2d_gb300.h and the reference signatures of
include/NFFT2_2D.cuh / NDFT2_2D.cuh, and validates arguments on the host."""
import ctypes
import os
import re
import subprocess

import pytest

from miscellaneous_gb300 import _lib


def test_library_exports_every_header_function(lib):
    names = _lib.header_functions()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_signatures_are_exported(lib):
    # Itanium mangling of the reference's C++ overloads (NFFT/NFFT2_2D.cuh:4-11)
    # and the extern "C" NDFT2_2D_GPU (NFFT/NDFT2_2D.cuh:4-6).
    for sym in ["NDFT2_2D_GPU",
                "_Z12NFFT2_2D_GPUP6float2PKS_PKfS4_iii",
                "_Z12NFFT2_2D_GPUP7double2PKS_PKdS4_iii",
                "_Z33Calculate_cuFFT_plan_C2C_NFFT2_2Dii",
                "_Z33Calculate_cuFFT_plan_Z2Z_NFFT2_2Dii",
                "_Z27Destroy_cuFFT_plan_NFFT2_2Dv",
                "NFFT2_2D_GPUplan"]:
        assert hasattr(lib, sym), sym


def test_compat_headers_compile_as_a_reference_caller():
    """A translation unit that includes both compat headers and calls every
    reference entry point must compile as plain C++ (host compiler only)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = r'''
#include "NFFT2_2D.cuh"
#include "NDFT2_2D.cuh"
void f(float2* r, const float2* d, const float* x, const float* y,
       double2* rd, const double2* dd, const double* xd, const double* yd, double2_* o) {
    Calculate_cuFFT_plan_C2C_NFFT2_2D(8, 8);
    NFFT2_2D_GPU(r, d, x, y, 8, 8, 3);
    Calculate_cuFFT_plan_Z2Z_NFFT2_2D(8, 8);
    NFFT2_2D_GPU(rd, dd, xd, yd, 8, 8, 3);
    NDFT2_2D_GPU(nullptr, xd, yd, xd, yd, o, o, 8, 8, 3, 3);
    Destroy_cuFFT_plan_NFFT2_2D();
    (void)NFFT2_2D_GPUplan;
}
'''
    cuda_inc = "/usr/local/cuda/include"
    if not os.path.isdir(cuda_inc):
        pytest.skip("CUDA headers not present")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-x", "c++", "-", "-I", os.path.join(root, "include"),
                        "-I", cuda_inc], input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_status_strings(lib):
    for code in range(0, -12, -1):
        s = _lib.status_string(code)
        assert s and s != "unknown status"
    assert _lib.status_string(-999) == "unknown status"


def test_layout_query_host_only(lib):
    info = _lib.Info()
    assert lib.nfft2d_layout_query(512, 512, 2.0, 6, 0, 0, ctypes.byref(info)) == 0
    d = info.as_dict()
    assert (d["n1"], d["n2"]) == (1024, 1024)
    # default 16 x 16 tiles; rows: whole tiles + halo; pitch: + patch pitch pad
    assert d["tile"] == 16 and (d["tiles1"], d["tiles2"]) == (64, 64)
    # 28 columns needed, pitch rounded up to 16 complex, plus the strip width
    # (4 at K = 6) so that the rows of a strip-ordered tile meet distinct banks
    assert (d["patch_rows"], d["patch_cols"]) == (28, 36)
    assert d["halo"] == 8 and (d["rows"], d["cols"]) == (1040, 1024 + 16 + 36 - 28)
    assert lib.nfft2d_layout_query(512, 512, 2.0, 6, 0, 32, ctypes.byref(info)) == 0
    assert (info.patch_rows, info.patch_cols, info.cols) == (44, 48, 1044)  # 32 x 32 tiles: row-major, no shift
    assert lib.nfft2d_layout_query(22, 22, 2.0, 6, 0, 0, ctypes.byref(info)) == 0
    assert (info.rows, info.cols, info.tiles1) == (3 * 16 + 16, 3 * 16 + 16 + 8, 3)
    # odd K: patch columns are rounded up so every TMA x coordinate is 16-byte aligned
    assert lib.nfft2d_layout_query(64, 64, 2.0, 5, 0, 16, ctypes.byref(info)) == 0
    assert info.patch_cols == 32 + 4 and info.patch_rows == 16 + 10  # 16 + 12 -> 32, + strip width 4
    assert lib.nfft2d_layout_query(64, 64, 2.0, 8, 0, 16, ctypes.byref(info)) == 0
    assert info.patch_cols == 32  # K = 8: one strip per tile, plain row-major order
    # the reference test's grid (22 -> 44) gets a partial last tile
    assert lib.nfft2d_layout_query(22, 22, 2.0, 6, 0, 0, ctypes.byref(info)) == 0
    assert info.n1 == 44 and info.tile == 16 and info.tiles1 == 3


@pytest.mark.parametrize("args", [
    (63, 64, 2.0, 6, 0, 0),     # odd N
    (64, 64, 2.0, 1, 0, 0),     # K too small
    (64, 64, 2.0, 9, 0, 0),     # K too large
    (64, 64, 1.0, 6, 0, 0),     # sigma < 1.25
    (64, 64, 1.3, 6, 0, 0),     # sigma*N not an integer
    (10, 10, 1.5, 6, 0, 0),     # sigma*N odd (15)
    (8, 8, 1.5, 6, 0, 0),       # sigma*N < 2K+2
    (64, 64, 2.0, 6, 2, 0),     # bad precision
    (64, 64, 2.0, 6, 0, 24),    # bad tile
    (8, 8, 2.0, 6, 0, 32),      # tile larger than the grid
])
def test_layout_query_rejects_bad_arguments(lib, args):
    info = _lib.Info()
    assert lib.nfft2d_layout_query(*args, ctypes.byref(info)) == _lib.ERR_INVALID_ARG


def test_plan_create_validates_before_touching_the_device(lib):
    h = ctypes.c_void_p()
    assert lib.nfft2d_plan_create(ctypes.byref(h), 63, 64, 2.0, 6, 0, None) == _lib.ERR_INVALID_ARG
    assert not h.value
    assert lib.nfft2d_plan_create(None, 64, 64, 2.0, 6, 0, None) == _lib.ERR_INVALID_ARG


def test_null_plan_is_rejected(lib):
    assert lib.nfft2d_plan_destroy(None) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_set_points(None, 0, None, None, 0, 0) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_forward(None, None, None) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_adjoint(None, None, None) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_synchronize(None) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_ndft2d_f64(None, None, None, None, None, None, 0, 8, 1, 1, -1, None) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_ndft2d_f64(None, None, None, None, None, None, 8, 8, 0, 0, -1, None) == 0


def test_batch_create_validates_before_touching_the_device(lib):
    h = ctypes.c_void_p()
    n1 = (ctypes.c_int * 3)(64, 32, 48)
    n2 = (ctypes.c_int * 3)(64, 32, 48)
    for ks in ((6, 1, 6), (6, 9, 6)):  # a half-width outside 2..8
        k = (ctypes.c_int * 3)(*ks)
        assert lib.nfft2d_batch_create_k(ctypes.byref(h), 3, n1, n2, k, 2.0, None) == _lib.ERR_INVALID_ARG
    k = (ctypes.c_int * 3)(6, 3, 8)
    assert lib.nfft2d_batch_create_k(ctypes.byref(h), 0, n1, n2, k, 2.0, None) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_batch_create_k(ctypes.byref(h), 3, n1, n2, None, 2.0, None) == _lib.ERR_INVALID_ARG
    odd = (ctypes.c_int * 3)(64, 33, 48)
    assert lib.nfft2d_batch_create_k(ctypes.byref(h), 3, odd, n2, k, 2.0, None) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_batch_create(ctypes.byref(h), 3, odd, n2, 2.0, 6, None) == _lib.ERR_INVALID_ARG
    assert not h.value
    assert lib.nfft2d_set_points_async(None, 0, None, None, 0, 0) == _lib.ERR_INVALID_ARG


def test_python_batch_rejects_mismatched_widths():
    import pytest as _pt
    from miscellaneous_gb300.nfft import Batch
    with _pt.raises(ValueError):
        Batch([(64, 64), (32, 32)], K=[6, 4, 8], stream=object())


def test_no_gpu_plan_create_reports_cuda_error(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    h = ctypes.c_void_p()
    st = lib.nfft2d_plan_create(ctypes.byref(h), 64, 64, 2.0, 6, 0, None)
    assert st == _lib.ERR_CUDA and not h.value


def test_package_fails_loudly_without_library(monkeypatch, tmp_path):
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load()


@pytest.mark.parametrize("T,B,N", [(0.25, 1.8, 24), (0.1, 4.5, 64), (0.3, 0.5 / 0.3, 160), (1.0, 0.5, 512)])
def test_knab_window_host_matches_oracle(lib, orc, T, B, N):
    # nfft2d_knab_window is host FP64 (Gauss-Legendre in theta), the oracle
    # restates MATLAB's adaptive Simpson quad at 1e-12: equal kg, G within
    # the oracle's quadrature tolerance
    from miscellaneous_gb300 import knab
    G, kg = knab.KnabWindow(T, B, 18, N)
    Go, kgo = orc.knab_window(T, B, 18, N)
    assert kg == kgo
    assert abs(G - Go).max() * N < 2e-12


def test_knab_window_rejects_bad_parameters(lib):
    kg = ctypes.c_int()
    for T, B, N in [(0.0, 1.0, 16), (0.5, 0.0, 16), (0.5, 2.5, 16), (0.5, 1.0, 0)]:
        assert lib.nfft2d_knab_window(T, B, 18, N, None, 0, ctypes.byref(kg)) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_knab_window(0.5, 1.0, 18, 16, None, 0, ctypes.byref(kg)) == 0
    G = (ctypes.c_double * 3)()
    # a buffer shorter than 2 kg + 1 is refused
    assert lib.nfft2d_knab_window(0.5, 1.0, 18, 16, G, 3, ctypes.byref(kg)) == _lib.ERR_INVALID_ARG
