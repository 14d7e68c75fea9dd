"""The reflectarray PSO far-field step for a swarm of particles
(nfft2d_batch_far_field; Synthesis/PSO/Synthesis.cu:385-405 around the
reference's per-particle NFFT2_2D_GPU call), at the reference's sizes
(kernel_single_v2.cu: 44 x 44 elements, 14.25 GHz, chi' = 4, so Nu = Nv = 44
and an 88 x 88 far field), with seeded aperiodic element positions and
excitations.

Checked per particle against the exact FP64 type-1 sum at the FP32-scaled
coordinates, times the visible-region filter (rel-L2 <= 1e-5, the FP32
bar), and one particle against the reference's own NFFT2_2D_GPU kernels
(oracle/_ref, the same FP32 inputs; rel-L2 <= 1e-5)."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FREQ = 14.25e9
LAM_F = float(np.float32(3e8 / FREQ))
LAM = 3e8 / FREQ
M_X = M_Y = 44


def _setup(particles=12, seed=9):
    from miscellaneous_gb300.nfft import pso_far_field_scales, pso_spectral_grid
    aap = float(np.float32((M_X - 1) * (LAM * 0.5 / 2.0)))        # kernel_single_v2.cu:39
    a_prime_f = float(np.float32(4 * aap))                        # :77
    beta = 2 * math.pi / LAM                                      # :27
    Nu, Nv = pso_spectral_grid(beta / 2, beta / 2, 4 * (M_X - 1) * (LAM * 0.5 / 2), 4 * (M_Y - 1) * (LAM * 0.5 / 2))
    sx, sy = pso_far_field_scales(Nu, Nv, a_prime_f, a_prime_f)
    rng = np.random.default_rng(seed)
    gx, gy = np.meshgrid((np.arange(M_X) - (M_X - 1) / 2) * 0.6 * LAM, (np.arange(M_Y) - (M_Y - 1) / 2) * 0.6 * LAM)
    X, Y, E = [], [], []
    for _ in range(particles):
        X.append((gx + rng.uniform(-0.05, 0.05, gx.shape) * LAM).ravel().astype(np.float32))
        Y.append((gy + rng.uniform(-0.05, 0.05, gy.shape) * LAM).ravel().astype(np.float32))
        E.append(np.exp(1j * rng.uniform(-math.pi, math.pi, gx.size)).astype(np.complex64))
    # visible-region filter on the 2Nv x 2Nu spectral grid (Synthesis.cu:71-106)
    u = (np.arange(-Nu, Nu) * (math.pi / (4 * (M_X - 1) * LAM * 0.25)))
    v = (np.arange(-Nv, Nv) * (math.pi / (4 * (M_Y - 1) * LAM * 0.25)))
    V, U = np.meshgrid(v, u, indexing="ij")
    filt = (U * U + V * V <= beta * beta).astype(np.float32)
    return Nu, Nv, sx, sy, X, Y, E, filt


def test_far_field_batch_matches_exact_and_reference_gpu(orc):
    from miscellaneous_gb300.nfft import Batch
    from oracle import ref_gpu
    Nu, Nv, sx, sy, X, Y, E, filt = _setup()
    dev = "cuda:0"
    n1, n2 = 2 * Nv, 2 * Nu
    tX = [torch.from_numpy(a).to(dev) for a in X]
    tY = [torch.from_numpy(a).to(dev) for a in Y]
    tE = [torch.from_numpy(a).to(dev) for a in E]
    tf = torch.from_numpy(filt.ravel()).to(dev)
    with Batch([(n1, n2)] * len(X), sigma=2.0, K=6) as b:
        outs = b.far_field(tX, tY, tE, sx, sy, tf)
        b.synchronize()
        got = [o.cpu().numpy().reshape(n1, n2) for o in outs]
        outs2 = b.far_field(tX[::-1], tY[::-1], tE[::-1], sx, sy, tf)  # new points, same batch
        b.synchronize()
        got2 = [o.cpu().numpy().reshape(n1, n2) for o in outs2]
    for p in range(len(X)):
        xs = (X[p] * np.float32(sx)).astype(np.float64)   # the FP32 scaling of :388-389
        ys = (Y[p] * np.float32(sy)).astype(np.float64)
        exact = orc.ndft_type1(E[p].astype(np.complex128), xs, ys, n1, n2, sign=-1) * filt
        assert orc.rel_l2(got[p], exact) < 1e-5, p
        np.testing.assert_allclose(got2[len(X) - 1 - p], got[p], rtol=0, atol=1e-3 * np.abs(got[p]).max())
    if ref_gpu.available():
        xs = torch.from_numpy((X[0] * np.float32(sx)).astype(np.float32)).to(dev)
        ys = torch.from_numpy((Y[0] * np.float32(sy)).astype(np.float32)).to(dev)
        ref = ref_gpu.nfft2_2d_gpu(tE[0], xs, ys, n1, n2).cpu().numpy() * filt
        assert orc.rel_l2(got[0], ref) < 1e-5
