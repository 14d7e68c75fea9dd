"""Coordinates in host memory: set_points reads page-locked host arrays over
the host link inside the binning pass (no separate upload), and the binned
state is identical to the one built from device copies of the same arrays.
Other host memory is read only where the device reports pageable-memory
access, and refused with NFFT2D_ERR_INVALID_ARG elsewhere."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def _inputs(dtype, M=70001, N=128, seed=21):
    g = torch.Generator().manual_seed(seed)
    x1 = (torch.rand(M, generator=g, dtype=torch.float64) - 0.5).to(dtype)
    x2 = (torch.rand(M, generator=g, dtype=torch.float64) - 0.5).to(dtype)
    F = torch.randn(N * N, dtype=torch.complex64, generator=g).to(DEV)
    f = torch.randn(M, dtype=torch.complex64, generator=g).to(DEV)
    return x1, x2, F, f, N


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_pinned_coordinates_match_device_coordinates(dtype):
    from miscellaneous_gb300.nfft import Plan
    x1, x2, F, f, N = _inputs(dtype)
    with Plan(N, N) as p:
        p.set_points(x1.to(DEV), x2.to(DEV))
        a_f, a_F = p.forward(F).clone(), p.adjoint(f).clone()
        info_dev = p.info()
        p.set_points(x1.pin_memory(), x2.pin_memory())
        b_f, b_F = p.forward(F).clone(), p.adjoint(f).clone()
        info_host = p.info()
        p.synchronize()
    assert info_dev["n_chunks"] == info_host["n_chunks"]
    torch.testing.assert_close(b_f, a_f, rtol=0, atol=0)  # same bins, same deterministic gather
    # the spread's tile reductions land in a run-dependent order: FP32 rounding only
    assert (torch.linalg.vector_norm(b_F - a_F) / torch.linalg.vector_norm(a_F)).item() < 1e-6


def test_unpinned_cpu_tensor_is_refused_by_the_wrapper():
    from miscellaneous_gb300.nfft import Plan
    x1, x2, _, _, N = _inputs(torch.float32, M=100)
    with Plan(N, N) as p:
        with pytest.raises(TypeError):
            p.set_points(x1, x2)


def test_pageable_host_pointer_is_read_or_refused():
    """Through the C ABI with a plain (pageable) host array: either the
    device can read pageable memory and the result equals the device-array
    run, or the call is refused with INVALID_ARG -- never a faulting read."""
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import Plan
    x1, x2, F, _, N = _inputs(torch.float32, M=5000)
    h1, h2 = x1.numpy().copy(), x2.numpy().copy()  # ordinary heap memory
    with Plan(N, N) as p:
        p.set_points(x1.to(DEV), x2.to(DEV))
        ref = p.forward(F).clone()
        p.synchronize()
        lib = _lib.load()
        st = lib.nfft2d_set_points(p._h, h1.size, ctypes.c_void_p(h1.ctypes.data), ctypes.c_void_p(h2.ctypes.data),
                                   _lib.COORD_F32, _lib.UNITS["unit"])
        assert st in (_lib.OK, _lib.ERR_INVALID_ARG)
        if st == _lib.OK:
            p.M = h1.size
            out = p.forward(F).clone()
            p.synchronize()
            torch.testing.assert_close(out, ref, rtol=0, atol=0)
