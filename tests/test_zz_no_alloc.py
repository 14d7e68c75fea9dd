"""nfft2d_forward_small_noalloc: the forward transform for callers that may
not allocate device memory while they run (a host that owns every device
allocation through its own pool, such as a MEX gateway working on gpuArray
data, or a latency-critical loop that cannot take cudaMalloc's implicit
synchronisation).  Its work buffers live in one fixed device array inside
the library instead of memory it allocates.

Checked through the C ABI against the existing plan entry point
nfft2d_forward on the same inputs, on two calls in a row (the second with
different inputs, so stale contents of the shared array would show), and
against the FP64 NDFT, in grid, unit and radian coordinates.  Tolerance:
rel-L2 <= 1e-5, the bar the other FP32 tests use against the FP64 NDFT.
After a first call has loaded the kernels, further calls leave the device's
free memory and torch's allocation count unchanged.  This file is collected
last on purpose.
"""
import ctypes
import gc

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _case(N1, N2, M, seed, units="unit"):
    rng = np.random.default_rng(seed)
    F = (rng.standard_normal((N1, N2)) + 1j * rng.standard_normal((N1, N2))).astype(np.complex64)
    x1 = rng.uniform(-0.5, 0.5, M).astype(np.float32)
    x2 = rng.uniform(-0.5, 0.5, M).astype(np.float32)
    if units == "grid":
        x1 = (x1 * N1).astype(np.float32)
        x2 = (x2 * N2).astype(np.float32)
    elif units == "radians":
        x1 = (x1 * 2 * np.pi).astype(np.float32)
        x2 = (x2 * 2 * np.pi).astype(np.float32)
    return F, x1, x2


def _grid_units(x, N, units):
    x = x.astype(np.float64)
    return {"grid": x, "unit": x * N, "radians": x * N / (2 * np.pi)}[units]


def _noalloc(lib, N1, N2, K, F, x1, x2, units):
    from miscellaneous_gb300 import _lib
    dev = "cuda:0"
    tF = torch.from_numpy(F).to(dev)
    t1 = torch.from_numpy(x1).to(dev)
    t2 = torch.from_numpy(x2).to(dev)
    out = torch.full((x1.size,), complex("nan"), dtype=torch.complex64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.nfft2d_forward_small_noalloc(N1, N2, K, x1.size, _ptr(t1), _ptr(t2), _lib.UNITS[units], _ptr(tF),
                                          _ptr(out), stream)
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _plan_forward(N1, N2, K, F, x1, x2, units):
    from miscellaneous_gb300.nfft import Plan
    with Plan(N1, N2, sigma=2.0, K=K) as p:
        p.set_points(torch.from_numpy(x1).cuda(), torch.from_numpy(x2).cuda(), units=units)
        f = p.forward(torch.from_numpy(F).cuda())
        p.synchronize()
        return f.cpu().numpy()


@pytest.mark.parametrize("N1,N2,K,M,units", [(64, 48, 6, 3000, "unit"), (128, 128, 6, 20000, "grid"),
                                             (16, 32, 4, 777, "unit"), (32, 64, 5, 1500, "radians")])
def test_noalloc_forward_matches_plan_forward_twice(lib, orc, N1, N2, K, M, units):
    for call, seed in enumerate((100 + N1, 200 + N2)):  # two calls in a row, different inputs
        F, x1, x2 = _case(N1, N2, M, seed, units)
        got = _noalloc(lib, N1, N2, K, F, x1, x2, units)
        want = _plan_forward(N1, N2, K, F, x1, x2, units)
        assert np.all(np.isfinite(got)), f"call {call}"
        assert orc.rel_l2(got, want) < 1e-5, f"call {call}"
        g1, g2 = _grid_units(x1, N1, units), _grid_units(x2, N2, units)
        exact = orc.ndft_type2(F.astype(np.complex128), g1, g2, sign=-1)
        assert orc.rel_l2(got, exact) < 1e-5, f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    from miscellaneous_gb300 import _lib
    z = ctypes.c_void_p(0)
    # grids larger than the fixed scratch: a clear, dedicated status
    assert lib.nfft2d_forward_small_noalloc(130, 64, 6, 0, z, z, 1, z, z, z) == _lib.ERR_SCRATCH_LIMIT
    assert lib.nfft2d_forward_small_noalloc(64, 256, 6, 0, z, z, 1, z, z, z) == _lib.ERR_SCRATCH_LIMIT
    # malformed requests
    assert lib.nfft2d_forward_small_noalloc(63, 64, 6, 0, z, z, 1, z, z, z) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_forward_small_noalloc(64, 64, 9, 0, z, z, 1, z, z, z) == _lib.ERR_INVALID_ARG
    assert lib.nfft2d_forward_small_noalloc(4, 4, 6, 0, z, z, 1, z, z, z) == _lib.ERR_INVALID_ARG
    assert "scratch" in _lib.status_string(_lib.ERR_SCRATCH_LIMIT)


def test_noalloc_call_allocates_no_device_memory(lib):
    """After a warm-up call (kernel loading may allocate once), a call leaves
    the device's free memory and torch's allocator untouched."""
    from miscellaneous_gb300 import _lib
    dev = "cuda:0"
    F, x1, x2 = _case(96, 96, 5000, 7)
    tF, t1, t2 = (torch.from_numpy(a).to(dev) for a in (F, x1, x2))
    out = torch.empty(x1.size, dtype=torch.complex64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call():
        st = lib.nfft2d_forward_small_noalloc(96, 96, 6, x1.size, _ptr(t1), _ptr(t2), _lib.UNITS["unit"], _ptr(tF),
                                              _ptr(out), stream)
        assert st == 0, _lib.status_string(st)
        torch.cuda.synchronize()

    call()
    # tensors of earlier tests that the cyclic collector frees in the middle
    # would change torch's count without any allocation by the call
    gc.collect()
    gc.disable()
    try:
        free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
        for _ in range(3):
            call()
        free1, alloc1 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    finally:
        gc.enable()
    assert free1 == free0
    assert alloc1 == alloc0
