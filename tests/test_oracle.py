"""Pins of the CPU oracle (no GPU): golden fixtures from the independent
numpy transliteration of the reference MATLAB files, the reference's own
acceptance test (Test_NFFT2_2D.m:24-29), analytic known answers, window
properties and the adjoint identity."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nfft_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def test_golden_reference_acceptance_case(orc, gold):
    # NFFT2_2D(data, y, x, M, N) of Test_NFFT2_2D.m:25 and NDFT2_2D(data, x, y, N, M) of :24
    a = orc.nfft2_2d(gold["reftest_data"], gold["reftest_y"], gold["reftest_x"], 22, 22)
    assert orc.rel_l2(a, gold["reftest_nfft"]) < 1e-13
    b = orc.ndft2_2d_matlab(gold["reftest_data"], gold["reftest_x"], gold["reftest_y"], 22, 22)
    assert orc.rel_l2(b, gold["reftest_ndft"]) < 1e-13
    # the reference prints 100*rel-L2 of NFFT vs NDFT (:28); the window's error is ~1e-11
    err_pct = 100 * orc.rel_l2(a, b)
    assert err_pct < 1e-8
    assert abs(err_pct - float(gold["reftest_err_pct"])) < 1e-9


def test_golden_forward_and_rectangular(orc, gold):
    f = orc.nfft1_2d(gold["fwd_F"], gold["fwd_x1"], gold["fwd_x2"])
    assert orc.rel_l2(f, gold["fwd_out"]) < 1e-13
    r = orc.nfft2_2d(gold["rect_d"], gold["rect_x1"], gold["rect_x2"], 16, 24)
    assert orc.rel_l2(r, gold["rect_out"]) < 1e-13


def test_exact_ndft_matches_matlab_layout(orc, gold):
    # type-1 exact sum with rows <-> y reproduces NDFT2_2D.m's N x M layout
    e = orc.ndft_type1(gold["reftest_data"], gold["reftest_y"], gold["reftest_x"], 22, 22, sign=-1)
    assert orc.rel_l2(e, gold["reftest_ndft"]) < 1e-13


def test_general_ndft_matches_exact(orc):
    rng = np.random.default_rng(1)
    N1, N2, M = 12, 10, 40
    x1 = (rng.random(M) - 0.5) * N1
    x2 = (rng.random(M) - 0.5) * N2
    d = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    k1, k2 = np.meshgrid(np.arange(N1) - N1 // 2, np.arange(N2) - N2 // 2, indexing="ij")
    out = orc.ndft2_2d_general(x1, x2, k1.ravel().astype(float), k2.ravel().astype(float), d, N1, N2)
    ref = orc.ndft_type1(d, x1, x2, N1, N2, sign=-1)
    assert orc.rel_l2(out, ref.ravel()) < 1e-13


def test_single_point_and_single_frequency_known_answers(orc):
    N = 16
    # one unit point at the origin spreads to all-ones coefficients
    F = orc.ndft_type1(np.array([1.0 + 0j]), np.array([0.0]), np.array([0.0]), N, N)
    assert np.allclose(F, 1.0, atol=1e-15)
    Fn = orc.nfft2_2d(np.array([1.0 + 0j]), np.array([0.0]), np.array([0.0]), N, N)
    assert np.allclose(Fn, 1.0, atol=1e-9)
    # a single frequency evaluates to a plane wave
    G = np.zeros((N, N), complex)
    G[N // 2 + 3, N // 2 - 5] = 1.0
    rng = np.random.default_rng(2)
    x1, x2 = (rng.random(30) - 0.5) * N, (rng.random(30) - 0.5) * N
    want = np.exp(-2j * np.pi * (3 * x1 / N - 5 * x2 / N))
    assert np.allclose(orc.ndft_type2(G, x1, x2), want, atol=1e-14)
    assert np.allclose(orc.nfft1_2d(G, x1, x2), want, atol=1e-9)


def test_shift_and_periodicity(orc):
    rng = np.random.default_rng(3)
    N = 16
    F = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    x1, x2 = (rng.random(25) - 0.5) * N, (rng.random(25) - 0.5) * N
    a = orc.nfft1_2d(F, x1, x2)
    b = orc.nfft1_2d(F, x1 + 3 * N, x2 - 2 * N)  # one period is N in grid units
    assert orc.rel_l2(a, b) < 1e-12


def test_adjoint_identity_exact(orc):
    rng = np.random.default_rng(4)
    N1, N2, M = 10, 14, 33
    F = rng.standard_normal((N1, N2)) + 1j * rng.standard_normal((N1, N2))
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    x1, x2 = (rng.random(M) - 0.5) * N1, (rng.random(M) - 0.5) * N2
    lhs = np.vdot(f, orc.ndft_type2(F, x1, x2, sign=-1))
    rhs = np.vdot(orc.ndft_type1(f, x1, x2, N1, N2, sign=+1), F)
    assert abs(lhs - rhs) < 1e-11 * abs(lhs)


def test_error_decreases_with_window_width(orc):
    rng = np.random.default_rng(5)
    N, M = 24, 200
    F = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    x1, x2 = (rng.random(M) - 0.5) * N, (rng.random(M) - 0.5) * N
    exact = orc.ndft_type2(F, x1, x2)
    errs = [orc.rel_l2(orc.nfft1_2d(F, x1, x2, K=K), exact) for K in range(2, 9)]
    assert all(b < a for a, b in zip(errs, errs[1:-1]))
    assert errs[4] < 1e-10  # K = 6


def test_window_pair_properties(orc):
    from scipy.special import i0
    K = 6
    a = orc.kb_alpha(2.0)
    assert a == pytest.approx(1.5 * np.pi - 0.01, abs=1e-15)
    for x in [0.0, 0.3, 5.0, 20.0, 28.2, 37.6]:
        assert orc.bessel_i0(x) == pytest.approx(float(i0(x)), rel=1e-14)
    # symmetric, alpha/pi at |t| = K, continuous across the sinh/sin switch
    for t in [0.1, 2.3, 5.9]:
        assert orc.phi_hat(t, K, a) == pytest.approx(orc.phi_hat(-t, K, a), rel=1e-15)
    assert orc.phi_hat(K, K, a) == pytest.approx(a / np.pi, rel=1e-15)
    assert orc.phi_hat(K - 1e-9, K, a) == pytest.approx(a / np.pi, rel=1e-6)
    assert orc.phi_hat(K + 1e-9, K, a) == pytest.approx(a / np.pi, rel=1e-6)
    # derivative vs central differences, both branches and at |t| = K
    h = 1e-6
    for t in [0.2, 3.7, 5.99999, 6.0, 6.3]:
        fd = (orc.phi_hat(t + h, K, a) - orc.phi_hat(t - h, K, a)) / (2 * h)
        assert orc.phi_hat_deriv(t, K, a) == pytest.approx(fd, rel=1e-5, abs=1e-6)


@pytest.mark.parametrize("shape", [(8, 16), (12, 10), (44, 44)])
def test_oracle_fft_matches_numpy(orc, shape):
    rng = np.random.default_rng(6)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    assert np.allclose(orc.fft2(a, -1), np.fft.fft2(a), atol=1e-11)
    assert np.allclose(orc.fft2(a, +1), np.fft.ifft2(a) * a.size, atol=1e-11)


def test_gradient_oracles(orc):
    rng = np.random.default_rng(7)
    N, M = 16, 40
    F = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    x1, x2 = (rng.random(M) - 0.5) * N, (rng.random(M) - 0.5) * N
    g1, g2 = orc.ndft_type2_grad(F, x1, x2)
    h = 1e-6
    fd1 = (orc.ndft_type2(F, x1 + h, x2) - orc.ndft_type2(F, x1 - h, x2)) / (2 * h)
    fd2 = (orc.ndft_type2(F, x1, x2 + h) - orc.ndft_type2(F, x1, x2 - h)) / (2 * h)
    assert orc.rel_l2(g1, fd1) < 1e-8 and orc.rel_l2(g2, fd2) < 1e-8
    a1, a2 = orc.nfft1_2d_grad(F, x1, x2)
    assert orc.rel_l2(a1, g1) < 1e-9 and orc.rel_l2(a2, g2) < 1e-9


def test_oracle_nfft1_1d_matches_direct_sum(orc):
    """Restated NFFT1_1D.m (c = 2, K = 6) against the exact 1D sum."""
    rng = np.random.default_rng(11)
    N = 216  # the reference's frequency samples per pulse (BP_FBP_FFBP_main.m:16)
    d = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    x = rng.uniform(-N / 2, N / 2, 300)
    k = np.arange(N) - N // 2
    exact = np.exp(-2j * np.pi * np.outer(x, k) / N) @ d
    assert orc.rel_l2(orc.nfft1_1d(d, x), exact) < 1e-10


def test_oracle_ffbp_focuses_a_point_target(orc):
    """The restated FFBP recursion images a point target at the scene centre,
    and a geometry with an odd NFFT grid is refused as the reference's
    NFFT1_2D would refuse it."""
    from oracle import ffbp as F
    data, sar = F.point_target_scene(Np=8, nf=64, Nx=32, R=2e3, step=0.08)
    im = np.nan_to_num(np.abs(F.ffbp(data, sar, 1, 8)))
    peak = np.unravel_index(np.argmax(im), im.shape)
    assert all(abs(p - 15.5) <= 1.5 for p in peak)
    data, sar = F.point_target_scene(Np=16, nf=64, Nx=32, R=2e3, step=0.08)
    with pytest.raises(ValueError):
        F.ffbp(data, sar, 1, 16)


def test_oracle_nufft3_matches_exact_sum(orc):
    """Restated NUFFT_2D_CPU (NFFT3_2D_C.cpp) against the exact type-3 sum at
    the accuracies asked for."""
    rng = np.random.default_rng(12)
    M, N = 1500, 1200
    x, y = rng.uniform(-3, 5, M), rng.uniform(-2, 2, M)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    s, t = rng.uniform(-20, 10, N), rng.uniform(-15, 15, N)
    exact = orc.ndft3_2d(x, y, f, s, t)
    for eps in (1e-4, 1e-8, 1e-12):
        F, info = orc.nufft3_2d(x, y, f, s, t, eps)
        assert info["Mrx"] % 2 == 0 and info["Mry"] % 2 == 0
        assert orc.rel_l2(F, exact) < max(eps, 1e-11)
