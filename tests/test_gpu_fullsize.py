"""Parity at the benchmark configurations' full sizes, through properties that
do not depend on the size: an exact FP64 NDFT on a random subset of the
points (torch complex128 on the GPU), the adjoint identity
<A F, f> = <F, A^H f>, agreement of the batched launch with single plans,
and a descent step of the least-squares loss.

Tolerances: FP32 plans vs the FP64 NDFT rel-L2 <= 1e-5 (the headline bar);
adjoint identity relative mismatch <= 1e-5 (FP32 accumulation over 2^24
points); batch vs single plans rel-L2 <= 1e-6.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def _ndft_subset(F, x1, x2, idx, sign):
    """Exact f_p = sum_k F_k exp(sign 2 pi i k.x_p) for the points idx
    (unit coordinates), FP64 phases reduced exactly, complex128 GEMMs."""
    N1, N2 = F.shape
    Fd = F.to(torch.complex128)

    def phases(x, N):
        k = torch.arange(N, device=DEV, dtype=torch.float64) - N // 2
        a = x.double()[:, None] * N * k[None, :] / N
        a = a - torch.round(a)
        return torch.exp(1j * (2 * math.pi * sign) * a)
    out = []
    for s in range(0, idx.numel(), 2048):
        i = idx[s:s + 2048]
        e1, e2 = phases(x1[i], N1), phases(x2[i], N2)
        out.append(((e2 @ Fd.T) * e1).sum(1))
    return torch.cat(out)


def _rel(a, b):
    a, b = a.to(torch.complex128), b.to(torch.complex128)
    return (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)).item()


@pytest.fixture(scope="module")
def clustered():
    """Config 3: 2048^2 coefficients, 2^24 points from a wrapped 2D Gaussian
    (sigma 0.15): NumPy PCG64, seed 3, the benchmark's own inputs."""
    rng = np.random.default_rng(3)
    M, N = 1 << 24, 2048
    x1 = np.mod(rng.normal(0.0, 0.15, M) + 0.5, 1.0) - 0.5
    x2 = np.mod(rng.normal(0.0, 0.15, M) + 0.5, 1.0) - 0.5
    F = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    f = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    return t(x1.astype(np.float32)), t(x2.astype(np.float32)), t(F), t(f)


@pytest.mark.parametrize("K", [4, 6, 8])
def test_clustered_full_size(clustered, K):
    from miscellaneous_gb300.nfft import Plan
    x1, x2, F, f = clustered
    N = F.shape[0]
    with Plan(N, N, sigma=2.0, K=K) as p:
        p.set_points(x1, x2)
        AF = p.forward(F.reshape(-1))
        AHf = p.adjoint(f).reshape(-1)
        p.synchronize()
    # the exact FP64 sum on a 65,536-point random subset (PCG64)
    idx = torch.from_numpy(np.random.default_rng(100 + K).choice(x1.numel(), 65536, replace=False)).to(DEV)
    assert _rel(AF[idx], _ndft_subset(F, x1, x2, idx, -1)) < 1e-5
    lhs = torch.vdot(f.to(torch.complex128), AF.to(torch.complex128))
    rhs = torch.vdot(AHf.to(torch.complex128), F.reshape(-1).to(torch.complex128))
    assert (abs(lhs - rhs) / abs(lhs)).item() < 1e-5


def test_uneven_batch_full_size():
    """Config 4: 64 transforms, N = 2^U{7..10}, M = floor(10^U(4, log10 4e6));
    the batched launch equals single-transform plans."""
    from miscellaneous_gb300.nfft import Batch, Plan
    rng = np.random.default_rng(3)
    sizes, Ms = [], []
    for _ in range(64):
        n = 2 ** int(rng.integers(7, 11))
        sizes.append((n, n))
        Ms.append(int(10 ** rng.uniform(4, math.log10(4e6))))
    g = torch.Generator(device=DEV).manual_seed(4)
    x1s = [torch.rand(m, device=DEV, generator=g) - 0.5 for m in Ms]
    x2s = [torch.rand(m, device=DEV, generator=g) - 0.5 for m in Ms]
    Fs = [torch.randn(a * b, dtype=torch.complex64, device=DEV, generator=g) for a, b in sizes]
    fs = [torch.randn(m, dtype=torch.complex64, device=DEV, generator=g) for m in Ms]
    batch = Batch(sizes)
    batch.set_points(x1s, x2s)
    outs_f = batch.forward(Fs)
    outs_F = batch.adjoint(fs)
    batch.synchronize()
    for t in range(0, 64, 7):
        with Plan(*sizes[t]) as p:
            p.set_points(x1s[t], x2s[t])
            rf = p.forward(Fs[t])
            rF = p.adjoint(fs[t]).reshape(-1)
            p.synchronize()
        assert _rel(outs_f[t], rf) < 1e-6
        assert _rel(outs_F[t].reshape(-1), rF) < 1e-6
    batch.close()


def test_least_squares_full_size():
    """Config 5: 1024^2, 2^22 uniform points.  The adjoint identity holds at
    that size, and one steepest-descent step on f with the exact line search
    lowers ||A f - y||^2 by the amount the quadratic model predicts."""
    from miscellaneous_gb300.nfft import Plan
    g = torch.Generator(device=DEV).manual_seed(5)
    N, M = 1024, 1 << 22
    x1 = torch.rand(M, device=DEV, generator=g) - 0.5
    x2 = torch.rand(M, device=DEV, generator=g) - 0.5
    f_true = torch.randn(N * N, dtype=torch.complex64, device=DEV, generator=g)
    F = torch.randn(N * N, dtype=torch.complex64, device=DEV, generator=g)
    noise = torch.randn(M, dtype=torch.complex64, device=DEV, generator=g) * (1e-3 / math.sqrt(2))
    with Plan(N, N) as p:
        p.set_points(x1, x2)
        y = p.forward(f_true) + noise
        r = p.forward(F) - y
        loss0 = float(torch.sum(torch.abs(r) ** 2))
        grad = p.adjoint(2.0 * r).reshape(-1)          # the gradient of the loss with respect to F
        Ag = p.forward(grad)
        t = float(torch.real(torch.vdot(Ag, r))) / float(torch.sum(torch.abs(Ag) ** 2))
        loss1 = float(torch.sum(torch.abs(p.forward(F - t * grad) - y) ** 2))
        lhs = torch.vdot(r.to(torch.complex128), Ag.to(torch.complex128))
        rhs = torch.vdot(p.adjoint(r).reshape(-1).to(torch.complex128), grad.to(torch.complex128))
        p.synchronize()
    predicted = loss0 - float(torch.real(torch.vdot(Ag, r))) ** 2 / float(torch.sum(torch.abs(Ag) ** 2))
    assert loss1 < loss0
    assert abs(loss1 - predicted) / loss0 < 1e-4
    assert (abs(lhs - rhs) / abs(lhs)).item() < 1e-5
