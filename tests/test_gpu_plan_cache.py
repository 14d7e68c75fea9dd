"""Plans made and dropped in turn reuse the library's cached resources (cuFFT
plans from the pool, device buffers from the block cache, page-locked
status slots).  Whatever a plan inherits, its results are the same as a
fresh plan's, on another stream too, and a plan whose FFT mode changes
takes the cuFFT plans of the new mode."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def _case(N, M, seed):
    g = torch.Generator(device=DEV).manual_seed(seed)
    x1 = torch.rand(M, device=DEV, generator=g) - 0.5
    x2 = torch.rand(M, device=DEV, generator=g) - 0.5
    F = torch.randn(N * N, dtype=torch.complex64, device=DEV, generator=g)
    f = torch.randn(M, dtype=torch.complex64, device=DEV, generator=g)
    return x1, x2, F, f


def _run(N, M, seed, stream=None, fft_mode=None):
    from miscellaneous_gb300.nfft import Plan
    x1, x2, F, f = _case(N, M, seed)
    with Plan(N, N, stream=stream) as p:
        if fft_mode is not None:
            p.set_tuning(fft_mode=fft_mode)
        p.set_points(x1, x2)
        a = p.forward(F).clone()
        b = p.adjoint(f).clone()
        p.synchronize()
    return a, b


def _rel(a, b):
    return (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)).item()


def test_reused_resources_give_the_same_results_on_another_stream(orc):
    # odd sizes: the cuFFT path (no fused passes); 90 x 90 -> a 180 x 180 grid
    shapes = [(90, 20000), (130, 50000), (90, 20000), (64, 8000), (130, 50000)]
    first = {}
    s2 = torch.cuda.Stream(device=DEV)
    for i, (N, M) in enumerate(shapes):
        stream = s2 if i % 2 else None
        with torch.cuda.stream(s2 if stream is not None else torch.cuda.current_stream()):
            a, b = _run(N, M, seed=N, stream=stream)
        torch.cuda.synchronize()
        if (N, M) in first:
            a0, b0 = first[(N, M)]
            torch.testing.assert_close(a, a0, rtol=0, atol=0)  # the gather is deterministic
            assert _rel(b, b0) < 1e-6                          # the spread's reduce order varies
        else:
            first[(N, M)] = (a, b)
    # and against the oracle for one of them
    N, M = 90, 20000
    x1, x2, F, f = _case(N, M, seed=N)
    want = orc.nfft1_2d(F.cpu().numpy().reshape(N, N).astype(np.complex128), x1.cpu().double().numpy() * N,
                        x2.cpu().double().numpy() * N, sign=-1)
    got = first[(N, M)][0].cpu().numpy().astype(np.complex128)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5


def test_fft_mode_change_takes_the_new_modes_plans():
    # 1024 x 1024 cells: fused passes by default (no cuFFT plan made);
    # cuFFT 2D (mode 0) and the pruned passes (mode 1) must give the same result
    N, M = 512, 100000
    a2, b2 = _run(N, M, seed=3)
    for mode in (0, 1):
        a, b = _run(N, M, seed=3, fft_mode=mode)
        assert _rel(a, a2) < 2e-6 and _rel(b, b2) < 2e-6, mode


def test_tuning_arguments_left_out_keep_their_settings():
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import Plan
    x1, x2, F, f = _case(256, 100000, seed=5)
    with Plan(256, 256) as p:
        p.set_tuning(gather_variant=_lib.VARIANT_TILED, chunk=256)
        p.set_points(x1, x2)
        p.set_tuning(io_order="binned")
        p.set_tuning(io_order="caller", fft_mode=0)
        info = p.info()
        assert info["gather_variant"] == _lib.VARIANT_TILED and info["chunk"] == 256 and info["fft_mode"] == 0
        # back to the automatic choice: 100,000 points on 32 x 32 tiles of 16^2 cells is
        # 98 points per tile, below the direct gather's 128
        p.set_tuning(gather_variant=_lib.VARIANT_AUTO)
        p.set_points(x1, x2)
        assert p.info()["gather_variant"] == _lib.VARIANT_TILED
