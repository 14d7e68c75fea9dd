"""The GPU path through the reference-named mirror functions
(miscellaneous_gb300.nfft.NFFT2_2D / NFFT1_2D / NDFT2_2D) against the golden
fixtures of tests/golden/nfft_golden.npz (numpy transliteration of the
reference MATLAB files), including the reference's own acceptance test
Test_NFFT2_2D.m:24-29.

Tolerances: FP32 vs the golden NFFT (same algorithm) rel-L2 <= 2e-6; FP32 vs
the golden NDFT <= 1e-5; FP64 vs golden NFFT <= 1e-12; FP64 NDFT <= 1e-13."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nfft_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def _t(a, dtype, dev="cuda:0"):
    return torch.from_numpy(np.ascontiguousarray(a).astype(dtype)).to(dev)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_reference_acceptance_test(orc, gold, prec):
    from miscellaneous_gb300 import nfft
    cdt = np.complex64 if prec == "f32" else np.complex128
    rdt = np.float32 if prec == "f32" else np.float64
    x, y, data = gold["reftest_x"], gold["reftest_y"], gold["reftest_data"]
    # Test_NFFT2_2D.m:25 -- NFFT2_2D(data, y, x, M, N)
    t2 = nfft.NFFT2_2D(_t(data, cdt), _t(y, rdt), _t(x, rdt), 22, 22).cpu().numpy()
    # Test_NFFT2_2D.m:24 -- NDFT2_2D(data, x, y, N, M)
    t1 = nfft.NDFT2_2D(_t(data, np.complex128), _t(x, np.float64), _t(y, np.float64), 22, 22).cpu().numpy()
    assert orc.rel_l2(t1, gold["reftest_ndft"]) < 1e-13
    if prec == "f32":
        # inputs rounded to FP32 move the points by ~1e-7 grid units
        assert orc.rel_l2(t2, gold["reftest_nfft"]) < 1e-5
        assert 100 * orc.rel_l2(t2, t1) < 1e-3  # the % figure Test_NFFT2_2D.m:28 prints
    else:
        assert orc.rel_l2(t2, gold["reftest_nfft"]) < 1e-12
        assert 100 * orc.rel_l2(t2, t1) < 1e-8


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_golden_forward_and_rectangular(orc, gold, prec):
    from miscellaneous_gb300 import nfft
    cdt = np.complex64 if prec == "f32" else np.complex128
    rdt = np.float32 if prec == "f32" else np.float64
    tol = 2e-6 if prec == "f32" else 1e-12
    # FP32: compare against the oracle at the FP32-rounded inputs (same algorithm)
    F, x1, x2 = gold["fwd_F"], gold["fwd_x1"].astype(rdt), gold["fwd_x2"].astype(rdt)
    f = nfft.NFFT1_2D(_t(F, cdt), _t(x1, rdt), _t(x2, rdt)).cpu().numpy()
    ref = gold["fwd_out"] if prec == "f64" else orc.nfft1_2d(F.astype(cdt), x1, x2)
    assert orc.rel_l2(f, ref) < tol
    d, r1, r2 = gold["rect_d"], gold["rect_x1"].astype(rdt), gold["rect_x2"].astype(rdt)
    r = nfft.NFFT2_2D(_t(d, cdt), _t(r1, rdt), _t(r2, rdt), 16, 24).cpu().numpy()
    ref = gold["rect_out"] if prec == "f64" else orc.nfft2_2d(d.astype(cdt), r1, r2, 16, 24)
    assert orc.rel_l2(r, ref) < tol


def test_nfft2_2d_gpu_mirror_in_place(orc, gold):
    from miscellaneous_gb300 import nfft
    x, y, data = gold["reftest_x"], gold["reftest_y"], gold["reftest_data"]
    res = torch.empty(22 * 22, dtype=torch.complex128, device="cuda:0")
    nfft.Calculate_cuFFT_plan_Z2Z_NFFT2_2D(22, 22)
    nfft.NFFT2_2D_GPU(res, _t(data, np.complex128), _t(y, np.float64), _t(x, np.float64), 22, 22, data.size)
    assert orc.rel_l2(res.cpu().numpy().reshape(22, 22), gold["reftest_nfft"]) < 1e-12
    nfft.Destroy_cuFFT_plan_NFFT2_2D()
