"""Parity against the reference's OWN GPU code.

oracle/build_ref.py compiles the reference's NFFT/NFFT2_2D.cu unchanged
(stand-in headers for the four it includes but does not ship) into a
device-linked sm_103a cubin; oracle/ref_harness.cpp restates the host side
of NFFT2_2D_GPU (NFFT2_2D.cu:329-495) and launches the reference's kernels
(Kernel_Bessel, Interpolation_NFFT2_2D_GPUKernel with its per-point child
grids of series_terms, fftshift + cuFFT, Decimation_and_Scaling).

Pins checked here, all at the reference's fixed sigma = 2, K = 6:
  * the golden fixtures (tests/golden/nfft_golden.npz, from the numpy
    transliteration of NFFT2_2D.m) agree with the reference's double
    overload to rel-L2 <= 1e-12;
  * the C oracle's restatement (oracle.nfft2_2d) agrees with it to <= 1e-12
    at config 1 (64 x 64, 4096 uniform points, seed 0);
  * the library's nfft2d_spread_ref (plan API and the NFFT2_2D_GPU shim)
    agrees with the reference's float overload to <= 1e-5 (both FP32; each
    is also checked against the exact FP64 sum) and with the double overload
    to <= 1e-12.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nfft_golden.npz")


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.fail("oracle/_ref/nfft2_2d_ref.cubin is missing: oracle.build_ref.build() must run where the "
                    "reference checkout is, and the cubin must travel with the repository")
    return ref_gpu


def _t(a, dtype, dev="cuda:0"):
    return torch.from_numpy(np.ascontiguousarray(a).astype(dtype)).to(dev)


def _config1(seed=0, N=64, M=4096):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.5, 0.5, M) * N
    y = rng.uniform(-0.5, 0.5, M) * N
    d = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
    return x, y, d


def test_golden_fixtures_match_reference_gpu(orc, ref):
    g = np.load(GOLDEN)
    # Test_NFFT2_2D.m:25 calls NFFT2_2D(data, y, x, M, N): y pairs with the rows
    out = ref.nfft2_2d_gpu(_t(g["reftest_data"], np.complex128), _t(g["reftest_y"], np.float64),
                           _t(g["reftest_x"], np.float64), 22, 22).cpu().numpy()
    assert orc.rel_l2(out, g["reftest_nfft"]) < 1e-12
    # and the acceptance figure that test prints (% rel-L2 vs the NDFT)
    assert 100 * orc.rel_l2(out, g["reftest_ndft"]) < 1e-8
    out = ref.nfft2_2d_gpu(_t(g["rect_d"], np.complex128), _t(g["rect_x1"], np.float64),
                           _t(g["rect_x2"], np.float64), 16, 24).cpu().numpy()
    assert orc.rel_l2(out, g["rect_out"]) < 1e-12
    out32 = ref.nfft2_2d_gpu(_t(g["rect_d"], np.complex64), _t(g["rect_x1"], np.float32),
                             _t(g["rect_x2"], np.float32), 16, 24).cpu().numpy()
    assert orc.rel_l2(out32, g["rect_out"]) < 1e-5


def test_oracle_restatement_matches_reference_gpu(orc, ref):
    x, y, d = _config1()
    out = ref.nfft2_2d_gpu(_t(d, np.complex128), _t(x, np.float64), _t(y, np.float64), 64, 64).cpu().numpy()
    assert orc.rel_l2(orc.nfft2_2d(d, x, y, 64, 64, sign=-1), out) < 1e-12
    exact = orc.ndft_type1(d, x, y, 64, 64, sign=-1)
    assert orc.rel_l2(out, exact) < 1e-10


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_library_spread_ref_matches_reference_gpu(orc, ref, prec):
    from miscellaneous_gb300 import nfft
    cdt, rdt = (np.complex64, np.float32) if prec == "f32" else (np.complex128, np.float64)
    x, y, d = _config1()
    xr, yr, dr = x.astype(rdt), y.astype(rdt), d.astype(cdt)
    out_ref = ref.nfft2_2d_gpu(_t(dr, cdt), _t(xr, rdt), _t(yr, rdt), 64, 64).cpu().numpy()
    with nfft.Plan(64, 64, sigma=2.0, K=6, precision=prec) as p:
        p.set_points(_t(xr, rdt), _t(yr, rdt), units="grid")
        ours = p.spread_ref(_t(dr, cdt)).cpu().numpy()
        p.synchronize()
    res = torch.empty(64 * 64, dtype=torch.complex64 if prec == "f32" else torch.complex128, device="cuda:0")
    nfft.NFFT2_2D_GPU(res, _t(dr, cdt), _t(xr, rdt), _t(yr, rdt), 64, 64, xr.size)
    shim = res.cpu().numpy().reshape(64, 64)
    nfft.Destroy_cuFFT_plan_NFFT2_2D()
    exact = orc.ndft_type1(dr.astype(np.complex128), xr.astype(np.float64), yr.astype(np.float64), 64, 64, sign=-1)
    tol = 1e-5 if prec == "f32" else 1e-12
    e_ours, e_ref = orc.rel_l2(ours, out_ref), orc.rel_l2(shim, out_ref)
    print(f"{prec}: library vs reference GPU {e_ours:.2e} (shim {e_ref:.2e}); vs exact: library "
          f"{orc.rel_l2(ours, exact):.2e}, reference {orc.rel_l2(out_ref, exact):.2e}")
    assert e_ours < tol and e_ref < tol
    assert orc.rel_l2(out_ref, exact) < (1e-5 if prec == "f32" else 1e-10)
    assert orc.rel_l2(ours, exact) < (1e-5 if prec == "f32" else 1e-10)


def test_reference_gpu_reference_acceptance_case_f32(orc, ref):
    """Test_NFFT2_2D.m's own shape (121 points, 22 x 22) with fresh seeded
    points, float overload against the library's FP32 NFFT2_2D mirror."""
    from miscellaneous_gb300 import nfft
    rng = np.random.default_rng(121)
    x = (11 * 0.5 * (rng.random(121) - 0.5)).astype(np.float32)
    y = (11 * 0.5 * (rng.random(121) - 0.5)).astype(np.float32)
    d = ((rng.random(121) - 0.5) + 1j * (rng.random(121) - 0.5)).astype(np.complex64)
    out_ref = ref.nfft2_2d_gpu(_t(d, np.complex64), _t(y, np.float32), _t(x, np.float32), 22, 22).cpu().numpy()
    ours = nfft.NFFT2_2D(_t(d, np.complex64), _t(y, np.float32), _t(x, np.float32), 22, 22).cpu().numpy()
    assert orc.rel_l2(ours, out_ref) < 1e-5
