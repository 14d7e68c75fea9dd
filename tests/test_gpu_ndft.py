"""The matrix-free FP64 direct sum (nfft2d_ndft2d_f64 / NDFT2_2D_GPU) against
the oracle's restatement of NDFT2_2D.cu at arbitrary frequencies.
Tolerance: rel-L2 <= 1e-12 (FP64, phases reduced before sincospi)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a).astype(dtype)).to("cuda:0")


@pytest.mark.parametrize("M,N", [(1, 1), (37, 300), (4096, 257), (129, 0), (0, 17)])
def test_ndft_general_frequencies(orc, M, N):
    from miscellaneous_gb300.nfft import NDFT2_2D_GPU
    rng = np.random.default_rng(M + N)
    Nu, Nv = 64, 48
    X = (rng.random(M) - 0.5) * Nu
    Y = (rng.random(M) - 0.5) * Nv
    u = rng.uniform(-Nu / 2, Nu / 2, N)       # arbitrary, non-integer frequencies
    v = rng.uniform(-Nv / 2, Nv / 2, N)
    d = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    out = torch.full((max(N, 1),), complex("nan"), dtype=torch.complex128, device="cuda:0")[:N]
    NDFT2_2D_GPU(_dev(X, np.float64), _dev(Y, np.float64), _dev(u, np.float64), _dev(v, np.float64),
                 _dev(d, np.complex128), out, Nu, Nv, M, N)
    torch.cuda.synchronize()
    if N == 0:
        return
    ref = orc.ndft2_2d_general(X, Y, u, v, d, Nu, Nv)
    got = out.cpu().numpy()
    if M == 0:
        assert np.all(got == 0)
        return
    assert orc.rel_l2(got, ref) < 1e-12


def test_ndft_sign_plus_is_conjugate_transform(orc):
    from miscellaneous_gb300.nfft import NDFT2_2D_GPU
    rng = np.random.default_rng(3)
    M, N = 200, 150
    X, Y = (rng.random(M) - 0.5) * 32, (rng.random(M) - 0.5) * 32
    u, v = rng.uniform(-16, 16, N), rng.uniform(-16, 16, N)
    d = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    out = torch.empty(N, dtype=torch.complex128, device="cuda:0")
    NDFT2_2D_GPU(_dev(X, np.float64), _dev(Y, np.float64), _dev(u, np.float64), _dev(v, np.float64),
                 _dev(np.conj(d), np.complex128), out, 32, 32, M, N, sign=+1)
    ref = np.conj(orc.ndft2_2d_general(X, Y, u, v, d, 32, 32))
    assert orc.rel_l2(out.cpu().numpy(), ref) < 1e-12
