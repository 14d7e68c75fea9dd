"""Type-3 2D NUFFT (nfft2d_nufft3_2d; NUFFT_2D_CPU of NFFT3_2D_C.cpp) on
the GPU against the oracle's restatement of the same Gaussian gridding and
against the exact sum F_k = sum_j f_j exp(-i (s_k x_j + t_k y_j)).

Tolerances: FP64 vs the restatement rel-L2 <= 1e-12 (same algorithm, same
parameters, different summation order); FP64 vs exact <= max(eps, 1e-11);
FP32 data (FP64 weights) vs exact <= 1e-5 at eps = 1e-6."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _case(seed, M=20000, N=15000):
    rng = np.random.default_rng(seed)
    x, y = rng.uniform(-40, 25, M), rng.normal(0, 6, M)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    s, t = rng.uniform(-3, 4, N), rng.uniform(-2.5, 2.5, N)
    return x, y, f, s, t


@pytest.mark.parametrize("eps", [1e-4, 1e-8, 1e-12])
def test_type3_f64_matches_restatement_and_exact(orc, eps):
    from miscellaneous_gb300.nufft3 import NUFFT_2D
    x, y, f, s, t = _case(31)
    got = NUFFT_2D(x, y, s, t, torch.tensor(f, dtype=torch.complex128), eps).cpu().numpy()
    ref, info = orc.nufft3_2d(x, y, f, s, t, eps)
    exact = orc.ndft3_2d(x, y, f, s, t)
    e_ref, e_ex = orc.rel_l2(got, ref), orc.rel_l2(got, exact)
    print(f"eps {eps:g} {info}: vs restatement {e_ref:.2e}, vs exact {e_ex:.2e}")
    assert e_ref <= 1e-12
    assert e_ex <= max(eps, 1e-11)


def test_type3_f32(orc):
    from miscellaneous_gb300.nufft3 import NUFFT_2D
    x, y, f, s, t = _case(32)
    got = NUFFT_2D(x, y, s, t, torch.tensor(f, dtype=torch.complex64), 1e-6).cpu().numpy()
    assert got.dtype == np.complex64
    assert orc.rel_l2(got, orc.ndft3_2d(x, y, f, s, t)) <= 1e-5


def test_type3_rejects_degenerate_extent():
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nufft3 import NUFFT_2D
    x = np.zeros(10)
    with pytest.raises(_lib.NFFT2DError) as e:
        NUFFT_2D(x, np.arange(10.0), np.arange(5.0), np.arange(5.0), torch.ones(10, dtype=torch.complex128), 1e-6)
    assert e.value.status == _lib.ERR_INVALID_ARG
