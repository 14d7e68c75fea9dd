"""miscellaneous_gb300 -- GB300-native (sm_103a) 2D NFFT with the call
surface of the reference's NFFT2_2D / NFFT1_2D / NDFT2_2D path.

The compute lives in ``lib/libnfft2d_gb300.so`` (hand-written CUDA kernels
plus cuFFT behind a C ABI, include/nfft2d_gb300.h).  This package binds it
with ctypes and uses PyTorch only for device memory and streams.
"""
from ._lib import NFFT2DError, LIB_PATH, load  # noqa: F401

__all__ = ["NFFT2DError", "LIB_PATH", "load", "nfft", "knab", "shard", "autotune"]


def __getattr__(name):
    # torch is imported lazily so the C-ABI checks run without it.
    if name in ("nfft", "shard", "knab", "autotune"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
