"""Failure handling, injected on the host or through bounded device waits --
nothing here faults, traps or hangs the GPU:

* every device allocation of plan creation and set_points fails in turn
  (NFFT2D_FAIL_ALLOC_AT, the plan's allocation hook): each call returns
  NFFT2D_ERR_OOM, nothing leaks, and a plan made afterwards is correct;
* the bounded device-side wait gives up on a barrier nothing completes and
  the library reports NFFT2D_ERR_DEVICE_TIMEOUT with the context intact.
"""
import ctypes
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _transform(N, x1, x2, F, f):
    from miscellaneous_gb300.nfft import Plan
    with Plan(N, N) as p:
        p.set_points(x1, x2)
        a = p.forward(F)
        b = p.adjoint(f)
        p.synchronize()
    return a, b


def test_every_allocation_failure_returns_oom_and_leaks_nothing():
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import Plan
    dev = "cuda:0"
    g = torch.Generator(device=dev).manual_seed(11)
    N, M = 64, 3000
    x1 = torch.rand(M, device=dev, generator=g) - 0.5
    x2 = torch.rand(M, device=dev, generator=g) - 0.5
    F = torch.randn(N * N, dtype=torch.complex64, device=dev, generator=g)
    f = torch.randn(M, dtype=torch.complex64, device=dev, generator=g)
    ref_a, ref_b = _transform(N, x1, x2, F, f)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failed_at = []
    try:
        for k in range(1, 40):
            os.environ["NFFT2D_FAIL_ALLOC_AT"] = str(k)
            try:
                with Plan(N, N) as p:
                    p.set_points(x1, x2)
                    p.synchronize()
            except _lib.NFFT2DError as e:
                assert e.status == _lib.ERR_OOM, (k, e.status)
                failed_at.append(k)
                continue
            break  # k is past the last allocation: everything succeeded
    finally:
        os.environ.pop("NFFT2D_FAIL_ALLOC_AT", None)
    assert len(failed_at) >= 8  # grid, tables, status, bins, records ...
    assert failed_at == list(range(1, len(failed_at) + 1))
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 < 64 << 20, (free0 - free1)  # no leaked plan buffers
    a, b = _transform(N, x1, x2, F, f)
    torch.testing.assert_close(a, ref_a, rtol=0, atol=0)  # the gather is deterministic
    # the spread's tile reductions land in a run-dependent order: FP32 rounding only
    assert (torch.linalg.vector_norm(b - ref_b) / torch.linalg.vector_norm(ref_b)).item() < 1e-6


def test_bounded_device_wait_reports_timeout():
    from miscellaneous_gb300 import _lib
    lib = _lib.load()
    s = torch.cuda.current_stream()
    st = lib.nfft2d_selftest_wait_timeout(1000, ctypes.c_void_p(s.cuda_stream))
    assert st == _lib.ERR_DEVICE_TIMEOUT
    assert lib.nfft2d_selftest_wait_timeout(0, ctypes.c_void_p(s.cuda_stream)) == _lib.ERR_INVALID_ARG
    # the context is intact: a transform still runs and agrees with the exact sum
    dev = "cuda:0"
    rng = np.random.default_rng(5)
    N, M = 32, 200
    x1 = rng.uniform(-0.5, 0.5, M).astype(np.float32).astype(np.float64)
    x2 = rng.uniform(-0.5, 0.5, M).astype(np.float32).astype(np.float64)
    F = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    k = np.arange(N) - N // 2
    exact = np.einsum("pi,ij,pj->p", np.exp(-2j * np.pi * np.outer(x1, k)), F, np.exp(-2j * np.pi * np.outer(x2, k)))
    a, _ = _transform(N, torch.tensor(x1, dtype=torch.float32, device=dev),
                      torch.tensor(x2, dtype=torch.float32, device=dev),
                      torch.tensor(F.reshape(-1), dtype=torch.complex64, device=dev),
                      torch.zeros(M, dtype=torch.complex64, device=dev))
    a = a.cpu().numpy()
    assert np.linalg.norm(a - exact) / np.linalg.norm(exact) < 1e-5  # the FP32 bar


def test_latched_timeout_is_reported_once_then_clears():
    """A bounded wait that runs out on a plan's (and a batch's) stream latches
    a timeout in its status word; the next synchronize reports it and clears
    it, so a correct run afterwards reports OK and gives right results."""
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import Batch, Plan
    lib = _lib.load()
    dev = "cuda:0"
    g = torch.Generator(device=dev).manual_seed(21)
    N, M = 32, 500
    x1 = torch.rand(M, device=dev, generator=g) - 0.5
    x2 = torch.rand(M, device=dev, generator=g) - 0.5
    F = torch.randn(N * N, dtype=torch.complex64, device=dev, generator=g)
    with Plan(N, N) as p:
        p.set_points(x1, x2)
        ref = p.forward(F)
        p.synchronize()
        assert lib.nfft2d_plan_selftest_wait_timeout(p.handle, 0) == _lib.ERR_INVALID_ARG
        assert lib.nfft2d_plan_selftest_wait_timeout(p.handle, 1000) == 0
        with pytest.raises(_lib.NFFT2DError) as e:
            p.synchronize()
        assert e.value.status == _lib.ERR_DEVICE_TIMEOUT
        out = p.forward(F)
        p.synchronize()  # reported once: a good run afterwards is OK
        torch.testing.assert_close(out, ref, rtol=0, atol=0)
    with Batch([(N, N), (16, 16)]) as b:
        b.set_points([x1, x1[:100].contiguous()], [x2, x2[:100].contiguous()])
        b.synchronize()
        assert lib.nfft2d_batch_selftest_wait_timeout(b._h, 1000) == 0
        with pytest.raises(_lib.NFFT2DError) as e:
            b.synchronize()
        assert e.value.status == _lib.ERR_DEVICE_TIMEOUT
        outs = b.forward([F, F[:256].contiguous()])
        b.synchronize()
        # batch (direct gather) vs plan (tiled gather): FP32 rounding only
        assert (torch.linalg.vector_norm(outs[0] - ref) / torch.linalg.vector_norm(ref)).item() < 1e-6


def test_huge_finite_coordinates_are_reduced_not_rejected():
    """A finite FP32 coordinate whose FP32 product with the (power-of-two)
    scale overflows is reduced in FP64 like any other; only NaN and +-Inf
    are rejected."""
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import Plan
    dev = "cuda:0"
    x1 = torch.tensor([0.1, 3.0e38, -2.5e38, 0.25], dtype=torch.float32, device=dev)
    x2 = torch.tensor([0.2, 0.3, 1.0e37, -0.4], dtype=torch.float32, device=dev)
    with Plan(16, 16) as p:
        p.set_points(x1, x2)  # units "unit": the scale sigma * N = 32 is a power of two; x * 32 overflows FP32
        F = torch.randn(256, dtype=torch.complex64, device=dev)
        f = p.forward(F)
        p.synchronize()
        assert torch.isfinite(torch.view_as_real(f)).all()
        with pytest.raises(_lib.NFFT2DError) as e:
            p.set_points(torch.tensor([0.1, float("inf")], device=dev), torch.tensor([0.0, 0.0], device=dev))
        assert e.value.status == _lib.ERR_NONFINITE
