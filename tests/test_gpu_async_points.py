"""nfft2d_set_points_async: binning without a host round trip.  The
transforms that follow read the work-item count from device memory and give
the same results as after the synchronous call; a non-finite coordinate is
reported by the next synchronize, and the transforms enqueued before that
stay in bounds."""
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def _inputs(M, N, seed):
    g = torch.Generator(device=DEV).manual_seed(seed)
    x1 = torch.rand(M, device=DEV, generator=g) - 0.5
    x2 = torch.rand(M, device=DEV, generator=g) - 0.5
    F = torch.randn(N * N, dtype=torch.complex64, device=DEV, generator=g)
    f = torch.randn(M, dtype=torch.complex64, device=DEV, generator=g)
    return x1, x2, F, f


def _rel(a, b):
    return (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)).item()


@pytest.mark.parametrize("gather_variant", [1, 2])
@pytest.mark.parametrize("N,M", [(64, 4096), (256, 200000)])
def test_async_matches_sync(N, M, gather_variant):
    from miscellaneous_gb300.nfft import Plan
    x1, x2, F, f = _inputs(M, N, seed=N)
    with Plan(N, N) as p:
        p.set_tuning(gather_variant=gather_variant)
        p.set_points(x1, x2)
        n_sync = p.info()["n_chunks"]
        a_f, a_F = p.forward(F).clone(), p.adjoint(f).clone()
        p.set_points(x1, x2, sync=False)
        assert p.info()["n_chunks"] == -1  # still on the device
        b_f, b_F = p.forward(F).clone(), p.adjoint(f).clone()
        p.synchronize()
        assert p.info()["n_chunks"] == n_sync
    torch.testing.assert_close(b_f, a_f, rtol=0, atol=0)
    assert _rel(b_F, a_F) < 1e-6  # tile reductions land in a run-dependent order


def test_async_nonfinite_reported_by_synchronize():
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import Plan
    N, M = 64, 5000
    x1, x2, F, f = _inputs(M, N, seed=9)
    bad = x1.clone()
    bad[123] = float("nan")
    bad[4000] = float("inf")
    with Plan(N, N) as p:
        p.set_points(bad, x2, sync=False)
        p.forward(F)   # enqueued before the status is read: runs in bounds
        p.adjoint(f)
        with pytest.raises(_lib.NFFT2DError) as e:
            p.synchronize()
        assert e.value.status == _lib.ERR_NONFINITE
        with pytest.raises(_lib.NFFT2DError) as e:
            p.forward(F)  # the point set was dropped
        assert e.value.status == _lib.ERR_NO_POINTS
        p.synchronize()  # the plan is usable again
        p.set_points(x1, x2, sync=False)
        out = p.forward(F)
        p.synchronize()
        p.set_points(x1, x2)
        ref = p.forward(F)
        p.synchronize()
    torch.testing.assert_close(out, ref, rtol=0, atol=0)


def test_automatic_gather_follows_bin_density():
    """The automatic FP32 gather is the tiled one on small, thin point sets
    and the direct one from 128 points per 16 x 16 tile (or 2^18 points) up,
    decided at set_points."""
    from miscellaneous_gb300.nfft import Plan
    N = 64  # 128^2 cells, 64 tiles
    with Plan(N, N) as p:
        x1, x2, _, _ = _inputs(4096, N, seed=1)       # 64 points per tile
        p.set_points(x1, x2)
        assert p.info()["gather_variant"] == 1
        x1, x2, _, _ = _inputs(64 * 256, N, seed=2)   # 256 points per tile
        p.set_points(x1, x2, sync=False)
        assert p.info()["gather_variant"] == 2
        p.set_tuning(gather_variant=1)                # an explicit choice sticks
        p.set_points(x1, x2)
        assert p.info()["gather_variant"] == 1
        p.synchronize()


@pytest.mark.parametrize("host_F", [False, True])
@pytest.mark.parametrize("host_coords", [False, True])
@pytest.mark.parametrize("N,M", [(64, 4096), (512, 300000), (1024, 100000)])
def test_bin_and_forward_matches_set_points_then_forward(N, M, host_coords, host_F):
    """nfft2d_bin_and_forward (the forward's padding and FFT on a second stream
    while the points are binned) gives the same result as set_points +
    forward, with device or page-locked host coordinates and F; its event
    marks the inputs read, and the adjoint that follows sees the new points."""
    from miscellaneous_gb300.nfft import Plan
    x1, x2, F, f = _inputs(M, N, seed=N + 1)
    with Plan(N, N) as p:
        p.set_points(x1, x2)
        want_f = p.forward(F).clone()
        want_F = p.adjoint(f).clone()
        p.synchronize()
        # other points first, so the call has to rebin
        y1, y2, _, _ = _inputs(M // 2 + 1, N, seed=7)
        p.set_points(y1, y2)
        c1, c2 = (x1.cpu().pin_memory(), x2.cpu().pin_memory()) if host_coords else (x1, x2)
        cF = F.cpu().pin_memory() if host_F else F
        ev = torch.cuda.Event()
        got_f = p.bin_and_forward(c1, c2, cF, inputs_read=ev)
        ev.synchronize()
        if host_F:
            cF.zero_()  # the inputs are read: rewriting the host F changes nothing
        got_F = p.adjoint(f)
        p.synchronize()
        torch.testing.assert_close(got_f, want_f, rtol=0, atol=0)  # same kernels, same order of sums
        assert _rel(got_F, want_F) < 1e-6                           # the spread's reduce order varies
        got0 = p.bin_and_forward(x1[:0], x2[:0], F.cpu().pin_memory() if host_F else F)
        p.synchronize()
        assert got0.numel() == 0
        if host_F:  # pageable host memory is refused
            with pytest.raises(TypeError):
                p.bin_and_forward(x1, x2, F.cpu())


@pytest.mark.parametrize("chunk", [256, 2048])
def test_large_work_items_with_asynchronous_binning(chunk):
    """Chunks above 512 points give the spread its own 512-point work list,
    whose count stays on the device: after an asynchronous binning (the
    combined call, page-locked host inputs) the forward and the adjoint equal
    those of a plan binned synchronously with the default work items."""
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import Plan
    N, M = 512, 400000
    x1, x2, F, f = _inputs(M, N, seed=21)
    with Plan(N, N) as ref:
        ref.set_points(x1, x2)
        want_f = ref.forward(F).clone()
        want_F = ref.adjoint(f).clone()
        ref.synchronize()
    with Plan(N, N) as p:
        p.set_tuning(chunk=chunk, gather_variant=_lib.VARIANT_TILED)
        got_f = p.bin_and_forward(x1.cpu().pin_memory(), x2.cpu().pin_memory(), F.cpu().pin_memory())
        got_F = p.adjoint(f)
        p.synchronize()
        assert p.info()["chunk"] == chunk and p.info()["n_chunks"] > 0
    assert _rel(got_f, want_f) < 1e-6  # tiled and direct gathers sum in different orders
    assert _rel(got_F, want_F) < 1e-6
