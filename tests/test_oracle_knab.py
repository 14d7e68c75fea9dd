"""Pins of the Knab-window regridding restatement in the CPU oracle (no GPU):
the golden fixture from the independent numpy transliteration of
BP_FBP_FFBP/knabNFFT2D.m, KnabWindow.m, ConvWindow.m and
NFFT_Based_Selvas_Approach_for_Signal_Interp_2D.m, the window's symmetry and
passband, and band-limited reproduction (the method's purpose)."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "knab_golden.npz")


@pytest.fixture(scope="module")
def kgold():
    return np.load(GOLDEN)


def test_knab_window_matches_golden(orc, kgold):
    G, kg = orc.knab_window(0.25, 1.8, 18, 24)
    assert kg == int(kgold["window_kg"])
    # adaptive Simpson (the oracle) vs QUADPACK (the fixture), both at 1e-12
    np.testing.assert_allclose(G, kgold["window_G"], rtol=0, atol=1e-13)


def test_knab_window_shape(orc):
    T, N = 0.1, 64
    B = 0.45 / T
    G, kg = orc.knab_window(T, B, 18, N)
    assert kg == int(np.floor((1 / T - B / 2) / (1 / (N * T))))
    np.testing.assert_allclose(G, G[::-1], rtol=0, atol=1e-15)       # KnabWindow.m:45 symmetry
    f = np.arange(-kg, kg + 1) / (N * T)
    inband = np.abs(f) <= B / 2 + 1e-12
    np.testing.assert_allclose(G[inband], 1.0 / N, rtol=0, atol=1e-15)  # G = 1/N in the signal band
    assert np.all(G >= -1e-15) and np.all(G <= 1.0 / N + 1e-15)
    # the roll-off decreases monotonically towards the edge of the window
    edge = G[:kg + 1][~inband[:kg + 1]]
    assert np.all(np.diff(edge) >= -1e-15)


def test_knab_regrid_matches_golden(orc, kgold):
    out, info = orc.knab_nfft2d(complex(kgold["extrap"]), kgold["rho_in"], kgold["cos_in"], kgold["data"],
                                kgold["rho_out"], kgold["cos_out"], float(kgold["B1"]), float(kgold["B2"]))
    assert (info["a"], info["b"], info["kgn"], info["kgm"]) == tuple(int(kgold[k]) for k in ("a", "b", "kgn", "kgm"))
    assert orc.rel_l2(out, kgold["out"]) < 1e-11
    ev = complex(kgold["extrap"])
    assert np.all(out[:, 0] == ev) and np.all(out[-1, :] == ev)


def test_knab_nfft_vs_direct_sum(orc, kgold):
    args = (complex(kgold["extrap"]), kgold["rho_in"], kgold["cos_in"], kgold["data"], kgold["rho_out"],
            kgold["cos_out"], float(kgold["B1"]), float(kgold["B2"]))
    a, _ = orc.knab_nfft2d(*args)
    b, _ = orc.knab_nfft2d(*args, direct=True)
    assert orc.rel_l2(a, b) < 1e-10  # NFFT1_2D's window error (c = 2, K = 6)


def _bandlimited(rho_in, cos_in, T1, T2):
    tones = [(0.2 / T1, -0.15 / T2, 1.0), (-0.1 / T1, 0.2 / T2, 0.5 + 0.3j), (0.05 / T1, 0.05 / T2, -0.7j)]

    def s(r, c):
        return sum(a * np.exp(2j * np.pi * (f1 * (r - rho_in[0]) + f2 * (c - cos_in[0]))) for f1, f2, a in tones)
    return s


@pytest.mark.parametrize("dense", [1, 3])
def test_knab_reproduces_bandlimited_signal(orc, dense):
    # away from the raster edges (more than P = 18 samples) the regridding is
    # exact for signals inside the band B = 0.5 / T, up to the window error
    Ncols, Nrows, T1, T2 = 128, 112, 0.3, 0.01
    rho_in = 100 + T1 * np.arange(Ncols)
    cos_in = -0.1 + T2 * np.arange(Nrows)
    s = _bandlimited(rho_in, cos_in, T1, T2)
    R, C = np.meshgrid(rho_in, cos_in)
    ro = np.linspace(rho_in[22], rho_in[-23], 84 * dense)
    co = np.linspace(cos_in[22], cos_in[-23], 68)
    RO, CO = np.meshgrid(ro, co)
    out, info = orc.knab_nfft2d(np.nan, rho_in, cos_in, s(R, C), RO, CO, 0.5 / T1, 0.5 / T2)
    assert info["a"] == max(2, round(RO.shape[1] / ((ro[-1] - ro[0]) / (T1 * (1 - 1 / RO.shape[1])))))
    assert orc.rel_l2(out, s(RO, CO)) < 1e-10
