"""GPU parity of the C-ABI transforms against the CPU oracle.

Tolerances (written per test):
  * FP32 plans vs the exact FP64 NDFT: rel-L2 <= 1e-5 (the bar of the
    headline metric) for K >= 4 at sigma = 2 -- the window error itself is
    5.6e-8 at K = 4 and 4.8e-12 at K = 6;
  * FP32 plans vs the restated reference algorithm with the same (sigma, K):
    rel-L2 <= 2e-6 (FP32 arithmetic only);
  * FP64 plans vs the restated reference algorithm: rel-L2 <= 1e-12.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _inputs(N1, N2, M, seed=0, dist="uniform"):
    rng = np.random.default_rng(seed)
    F = (rng.uniform(-1, 1, (N1, N2)) + 1j * rng.uniform(-1, 1, (N1, N2)))
    if dist == "uniform":
        x1 = rng.uniform(-0.5, 0.5, M)
        x2 = rng.uniform(-0.5, 0.5, M)
    elif dist == "cluster":
        x1 = np.mod(rng.normal(0, 0.02, M) + 0.5, 1.0) - 0.5
        x2 = np.mod(rng.normal(0, 0.02, M) + 0.5, 1.0) - 0.5
    else:
        raise ValueError(dist)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    return F, x1.astype(np.float32), x2.astype(np.float32), f


def _run(plan_kw, F, x1, x2, f, units="unit", dev="cuda:0", tuning=None):
    from miscellaneous_gb300.nfft import Plan
    N1, N2 = F.shape
    prec = plan_kw.get("precision", "f32")
    cdt = np.complex64 if prec == "f32" else np.complex128
    with Plan(N1, N2, **plan_kw) as p:
        if tuning:
            p.set_tuning(**tuning)
        xt1 = torch.from_numpy(np.ascontiguousarray(x1)).to(dev)
        xt2 = torch.from_numpy(np.ascontiguousarray(x2)).to(dev)
        p.set_points(xt1, xt2, units=units)
        Ft = torch.from_numpy(F.astype(cdt)).to(dev)
        ft = torch.from_numpy(f.astype(cdt)).to(dev)
        fwd = p.forward(Ft)
        adj = p.adjoint(ft)
        ref = p.spread_ref(ft)
        p.synchronize()
        return fwd.cpu().numpy(), adj.cpu().numpy(), ref.cpu().numpy(), p.info()


def _grid(x, N):
    return np.asarray(x, dtype=np.float64) * N


def test_config1_vs_exact_ndft(orc):
    """64x64, M = 4096 uniform, sigma = 2, w = 6: the reference-runnable case."""
    F, x1, x2, f = _inputs(64, 64, 4096, seed=0)
    fwd, adj, sref, info = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f)
    g1, g2 = _grid(x1, 64), _grid(x2, 64)
    e_fwd = orc.rel_l2(fwd, orc.ndft_type2(F, g1, g2, sign=-1))
    e_adj = orc.rel_l2(adj, orc.ndft_type1(f, g1, g2, 64, 64, sign=+1))
    e_ref = orc.rel_l2(sref, orc.ndft_type1(f, g1, g2, 64, 64, sign=-1))
    assert info["gather_variant"] == 1 and info["n_chunks"] > 0
    assert e_fwd < 1e-5, e_fwd
    assert e_adj < 1e-5, e_adj
    assert e_ref < 1e-5, e_ref


@pytest.mark.parametrize("K", [2, 3, 4, 5, 6, 7, 8])
def test_window_widths_vs_restated_algorithm(orc, K):
    F, x1, x2, f = _inputs(32, 48, 1500, seed=K)
    fwd, adj, sref, _ = _run({"sigma": 2.0, "K": K}, F, x1, x2, f)
    g1, g2 = _grid(x1, 32), _grid(x2, 48)
    a_fwd = orc.nfft1_2d(F, g1, g2, c=2.0, K=K, sign=-1)
    a_ref = orc.nfft2_2d(f, g1, g2, 32, 48, c=2.0, K=K, sign=-1)
    a_adj = orc.nfft2_2d(f, g1, g2, 32, 48, c=2.0, K=K, sign=+1)
    assert orc.rel_l2(fwd, a_fwd) < 2e-6
    assert orc.rel_l2(sref, a_ref) < 2e-6
    assert orc.rel_l2(adj, a_adj) < 2e-6
    if K >= 4:
        assert orc.rel_l2(fwd, orc.ndft_type2(F, g1, g2, sign=-1)) < 1e-5


@pytest.mark.parametrize("K", [3, 6, 8])
def test_f64_plan_vs_restated_algorithm(orc, K):
    F, x1, x2, f = _inputs(32, 32, 700, seed=10 + K)
    x1 = x1.astype(np.float64)
    x2 = x2.astype(np.float64)
    fwd, adj, sref, info = _run({"sigma": 2.0, "K": K, "precision": "f64"}, F, x1, x2, f)
    g1, g2 = _grid(x1, 32), _grid(x2, 32)
    assert orc.rel_l2(fwd, orc.nfft1_2d(F, g1, g2, K=K, sign=-1)) < 1e-12
    assert orc.rel_l2(sref, orc.nfft2_2d(f, g1, g2, 32, 32, K=K, sign=-1)) < 1e-12
    assert orc.rel_l2(adj, orc.nfft2_2d(f, g1, g2, 32, 32, K=K, sign=+1)) < 1e-12


@pytest.mark.parametrize("tile", [8, 16, 32, 64])
def test_tile_sizes_agree(orc, tile):
    F, x1, x2, f = _inputs(64, 64, 3000, seed=3, dist="cluster")
    fwd, adj, _, info = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f, tuning={"tile": tile, "chunk": 64})
    assert info["tile"] == tile
    g1, g2 = _grid(x1, 64), _grid(x2, 64)
    assert orc.rel_l2(fwd, orc.nfft1_2d(F, g1, g2, sign=-1)) < 2e-6
    assert orc.rel_l2(adj, orc.nfft2_2d(f, g1, g2, 64, 64, sign=+1)) < 2e-6


@pytest.mark.parametrize("chunk", [32, 100, 512, 4096])
def test_work_item_sizes_agree(orc, chunk):
    """The chunk is the tiled gather's patch item and the tiled spread's warp
    item: a tile's points cut at any size give the same transforms, from items
    of a few points to one item per dense tile."""
    F, x1, x2, f = _inputs(64, 64, 6000, seed=12, dist="cluster")
    fwd, adj, _, info = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f,
                             tuning={"chunk": chunk, "gather_variant": 1, "spread_variant": 1})
    assert info["chunk"] == chunk and info["gather_variant"] == 1 and info["spread_variant"] == 1
    g1, g2 = _grid(x1, 64), _grid(x2, 64)
    assert orc.rel_l2(fwd, orc.nfft1_2d(F, g1, g2, sign=-1)) < 2e-6
    assert orc.rel_l2(adj, orc.nfft2_2d(f, g1, g2, 64, 64, sign=+1)) < 2e-6


def test_direct_variant_matches_tiled(orc):
    F, x1, x2, f = _inputs(64, 32, 2000, seed=4)
    t = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f)
    d = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f, tuning={"gather_variant": 2, "spread_variant": 2})
    for a, b in zip(t[:3], d[:3]):
        assert orc.rel_l2(a, b) < 2e-6


def test_uncompensated_gather_still_within_bar(orc):
    F, x1, x2, f = _inputs(64, 64, 2000, seed=5)
    fwd, *_ = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f, tuning={"compensated": 0})
    assert orc.rel_l2(fwd, orc.ndft_type2(F, _grid(x1, 64), _grid(x2, 64), sign=-1)) < 1e-5


@pytest.mark.parametrize("N1,N2,sigma", [(22, 22, 2.0), (8, 8, 2.0), (16, 64, 2.0), (64, 64, 1.5), (48, 24, 1.25),
                                         (40, 80, 1.6), (96, 48, 4 / 3)])
def test_odd_shapes_and_oversampling(orc, N1, N2, sigma):
    """FP32 vs the restated algorithm: 2e-6 at sigma >= 1.5.  (40, 80, 1.6) and
    (96, 48, 4/3) land on power-of-two grids (64 x 128, 128 x 64), so the fused
    FFT passes run with band widths that are not multiples of the columns per
    CTA.  At sigma = 1.25
    (K = 5) the deapodization table spans I0(K alpha)/I0(K sqrt(alpha^2 -
    (pi/sigma)^2)) = I0(18.8)/I0(14.0) ~ 92x across the band, which scales
    FP32 rounding at the band edges by the same factor, so the bar there is 1e-4."""
    F, x1, x2, f = _inputs(N1, N2, 900, seed=N1 + N2)
    fwd, adj, sref, _ = _run({"sigma": sigma, "K": 5}, F, x1, x2, f)
    g1, g2 = _grid(x1, N1), _grid(x2, N2)
    tol = 2e-6 if sigma >= 1.5 else 1e-4  # sigma = 4/3: the deapodization spans ~46x across the band
    assert orc.rel_l2(fwd, orc.nfft1_2d(F, g1, g2, c=sigma, K=5, sign=-1)) < tol
    assert orc.rel_l2(sref, orc.nfft2_2d(f, g1, g2, N1, N2, c=sigma, K=5, sign=-1)) < tol
    assert orc.rel_l2(adj, orc.nfft2_2d(f, g1, g2, N1, N2, c=sigma, K=5, sign=+1)) < tol


def test_units_are_equivalent(orc):
    F, x1, x2, f = _inputs(32, 32, 1000, seed=6)
    u = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f, units="unit")
    g = _run({"sigma": 2.0, "K": 6}, F, (x1 * 32).astype(np.float32), (x2 * 32).astype(np.float32), f, units="grid")
    r = _run({"sigma": 2.0, "K": 6}, F, (x1.astype(np.float64) * 2 * np.pi), (x2.astype(np.float64) * 2 * np.pi),
             f, units="radians")
    for a, b, c in zip(u[:3], g[:3], r[:3]):
        assert orc.rel_l2(a, b) < 1e-6
        assert orc.rel_l2(a, c) < 1e-6


def test_edge_points_and_periodic_wrap(orc):
    N = 32
    x1 = np.array([-0.5, 0.5 - 2 ** -24, 0.0, 0.25, 1.25, -3.75, 0.49999, -0.49999], dtype=np.float32)
    x2 = np.array([0.0, -0.5, 0.5 - 2 ** -24, 2.25, -0.75, 0.125, -0.49999, 0.49999], dtype=np.float32)
    rng = np.random.default_rng(7)
    F = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    f = rng.standard_normal(x1.size) + 1j * rng.standard_normal(x1.size)
    fwd, adj, _, _ = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f)
    g1, g2 = _grid(x1, N), _grid(x2, N)
    assert orc.rel_l2(fwd, orc.ndft_type2(F, g1, g2, sign=-1)) < 1e-5
    assert orc.rel_l2(adj, orc.ndft_type1(f, g1, g2, N, N, sign=+1)) < 1e-5


def test_all_points_in_one_cell(orc):
    """Collisions: every point in the same oversampled cell."""
    M = 5000
    x1 = np.full(M, 0.1, dtype=np.float32) + np.float32(1e-4) * np.linspace(0, 1, M, dtype=np.float32)
    x2 = np.full(M, -0.2, dtype=np.float32)
    rng = np.random.default_rng(8)
    F = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    fwd, adj, _, info = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f)
    g1, g2 = _grid(x1, 64), _grid(x2, 64)
    assert info["n_chunks"] >= M // info["chunk"]
    assert orc.rel_l2(fwd, orc.nfft1_2d(F, g1, g2, sign=-1)) < 2e-6
    assert orc.rel_l2(adj, orc.nfft2_2d(f, g1, g2, 64, 64, sign=+1)) < 2e-6


@pytest.mark.parametrize("M", [0, 1, 31, 257])
def test_small_and_empty_point_sets(orc, M):
    F, x1, x2, f = _inputs(16, 16, M, seed=M)
    fwd, adj, sref, info = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f)
    assert fwd.shape == (M,)
    if M == 0:
        assert np.all(adj == 0) and np.all(sref == 0)
        return
    g1, g2 = _grid(x1, 16), _grid(x2, 16)
    assert orc.rel_l2(fwd, orc.nfft1_2d(F, g1, g2, sign=-1)) < 2e-6
    assert orc.rel_l2(adj, orc.nfft2_2d(f, g1, g2, 16, 16, sign=+1)) < 2e-6


def test_nonfinite_coordinate_is_rejected():
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import NFFT2DError, Plan
    x = torch.zeros(10, device="cuda:0")
    x[3] = float("nan")
    with Plan(16, 16) as p:
        with pytest.raises(NFFT2DError) as ei:
            p.set_points(x, torch.zeros(10, device="cuda:0"))
        assert ei.value.status == _lib.ERR_NONFINITE
        with pytest.raises(NFFT2DError) as ei:
            p.forward(torch.zeros(16 * 16, dtype=torch.complex64, device="cuda:0"))
        assert ei.value.status == _lib.ERR_NO_POINTS


def test_adjoint_identity_at_polar_scale():
    """<A F, f> == <F, A^H f> at the polar-raster size (512^2, 2^20 points)."""
    from miscellaneous_gb300.nfft import Plan
    g = torch.Generator(device="cuda:0").manual_seed(1)
    N, M = 512, 1 << 20
    x1 = torch.rand(M, device="cuda:0", generator=g) - 0.5
    x2 = torch.rand(M, device="cuda:0", generator=g) - 0.5
    F = torch.randn(N * N, dtype=torch.complex64, device="cuda:0", generator=g)
    f = torch.randn(M, dtype=torch.complex64, device="cuda:0", generator=g)
    with Plan(N, N) as p:
        p.set_points(x1, x2)
        AF = p.forward(F).to(torch.complex128)
        AHf = p.adjoint(f).reshape(-1).to(torch.complex128)
        p.synchronize()
    lhs = torch.vdot(f.to(torch.complex128), AF)       # <f, A F>
    rhs = torch.vdot(AHf, F.to(torch.complex128))       # <A^H f, F>
    rel = (abs(lhs - rhs) / abs(lhs)).item()
    assert rel < 1e-5, rel


def test_polar_raster_dense_centre(orc):
    """Polar raster (every spoke crosses the centre: hundreds of points per
    centre cell) at a size the oracle finishes quickly: 64 x 64 coefficients,
    64 spokes x 256 samples.  Exercises the spread's same-cell group path."""
    rng = np.random.default_rng(12)
    th = np.pi * np.arange(64) / 64
    r = -0.5 + np.arange(256) / 256
    R, TH = np.meshgrid(r, th, indexing="ij")
    x1 = (np.mod((R * np.cos(TH)).ravel() + rng.uniform(-1e-3, 1e-3, R.size) + 0.5, 1) - 0.5).astype(np.float32)
    x2 = (np.mod((R * np.sin(TH)).ravel() + rng.uniform(-1e-3, 1e-3, R.size) + 0.5, 1) - 0.5).astype(np.float32)
    F = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    f = rng.standard_normal(x1.size) + 1j * rng.standard_normal(x1.size)
    fwd, adj, sref, _ = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f)
    g1, g2 = _grid(x1, 64), _grid(x2, 64)
    assert orc.rel_l2(fwd, orc.nfft1_2d(F, g1, g2, sign=-1)) < 2e-6
    assert orc.rel_l2(adj, orc.nfft2_2d(f, g1, g2, 64, 64, sign=+1)) < 2e-6
    assert orc.rel_l2(sref, orc.nfft2_2d(f, g1, g2, 64, 64, sign=-1)) < 2e-6
    # repeated calls on the same plan give the same spread (patches are re-zeroed)
    adj2 = _run({"sigma": 2.0, "K": 6}, F, x1, x2, f)[1]
    assert orc.rel_l2(adj2, adj) < 1e-6


@pytest.mark.parametrize("N1,N2,sigma,prec,tol", [(64, 64, 2.0, "f32", 2e-6), (48, 24, 1.25, "f32", 5e-4),
                                                  (16, 64, 2.0, "f64", 1e-13), (512, 256, 2.0, "f32", 2e-6)])
def test_pruned_fft_matches_full_fft(N1, N2, sigma, prec, tol):
    """The two-pass FFT that skips the zero / cropped columns gives the same
    transforms as the plain 2D cuFFT plan, within FP32 rounding.  At
    sigma = 1.25 the deapodization amplifies the spread's rounding up to ~92x,
    and the spread's TMA reductions of overlapping strip patches land in a
    run-dependent order: two runs of the SAME FFT mode differ by up to
    2.2e-4 there (measured over 8 repetitions on GB300), so the bound sits
    above that."""
    F, x1, x2, f = _inputs(N1, N2, 3000, seed=21)
    kw = {"sigma": sigma, "K": 6, "precision": prec}
    a = _run(kw, F, x1, x2, f, tuning={"fft_mode": 1})
    b = _run(kw, F, x1, x2, f, tuning={"fft_mode": 0})
    for u, v in zip(a[:3], b[:3]):
        assert np.linalg.norm(u - v) / np.linalg.norm(v) < tol


@pytest.mark.parametrize("N1,N2,K", [(32, 32, 6), (64, 32, 4), (32, 512, 6), (512, 512, 6), (256, 1024, 8),
                                     (2048, 64, 3), (128, 2048, 6)])
def test_fused_fft_matches_cufft(N1, N2, K):
    """The library's own FFT passes fused with pad / halo fill / halo fold /
    crop (fft_mode 2, the default on power-of-two grids) give the same
    forward, adjoint and reference-sign spread as cuFFT's 2D plan around the
    separate stage kernels, to FP32 rounding (FFT sizes 64 .. 4096, square,
    tall and wide grids)."""
    F, x1, x2, f = _inputs(N1, N2, 5000, seed=N1 + N2)
    kw = {"sigma": 2.0, "K": K}
    a = _run(kw, F, x1, x2, f, tuning={"fft_mode": 2})
    b = _run(kw, F, x1, x2, f, tuning={"fft_mode": 0})
    for u, v in zip(a[:3], b[:3]):
        assert np.linalg.norm(u - v) / np.linalg.norm(v) < 2e-6


def test_fused_fft_mode_unsupported_off_power_of_two():
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import Plan
    with Plan(48, 24, sigma=1.25) as p:  # 60 x 30 oversampled cells
        with pytest.raises(_lib.NFFT2DError) as e:
            p.set_tuning(fft_mode=2)
        assert e.value.status == _lib.ERR_UNSUPPORTED
    with Plan(64, 64, precision="f64") as p:
        with pytest.raises(_lib.NFFT2DError) as e:
            p.set_tuning(fft_mode=2)
        assert e.value.status == _lib.ERR_UNSUPPORTED
