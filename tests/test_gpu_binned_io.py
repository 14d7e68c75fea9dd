"""Per-point arrays in the plan's binned order (nfft2d_tuning.io_order =
NFFT2D_ORDER_BINNED, nfft2d_get_permutation): the same transforms as the
caller's order, with f, v, g1, g2 permuted by perm -- bit for bit where the
arithmetic is the same (gather, gradient) and to FP32 rounding for the
adjoint (the spread adds the same terms; only the order of the TMA
reductions may differ), in both precisions and for both gather variants."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,variant", [("f32", 0), ("f32", 1), ("f32", 2), ("f64", 0)])
def test_binned_order_io_matches_caller_order(prec, variant):
    from miscellaneous_gb300.nfft import Plan
    dev = "cuda:0"
    rng = np.random.default_rng(77)
    N, M = 96, 20000
    cdt = torch.complex64 if prec == "f32" else torch.complex128
    rdt = torch.float32 if prec == "f32" else torch.float64
    x1 = torch.tensor(rng.normal(0, 0.2, M), dtype=rdt, device=dev)
    x2 = torch.tensor(rng.uniform(-0.5, 0.5, M), dtype=rdt, device=dev)
    F = torch.tensor(rng.standard_normal(N * N) + 1j * rng.standard_normal(N * N), dtype=cdt, device=dev)
    f = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), dtype=cdt, device=dev)
    with Plan(N, N, K=6, precision=prec) as p:
        if variant:
            p.set_tuning(gather_variant=variant)
        p.set_points(x1, x2)
        a_caller, A_caller = p.forward(F), p.adjoint(f)
        g_caller = p.grad_x(F, f)
        perm = p.permutation().long()
        p.synchronize()
        assert torch.equal(torch.sort(perm).values, torch.arange(M, device=dev))
        p.set_tuning(io_order="binned")
        a_binned, A_binned = p.forward(F), p.adjoint(f[perm].contiguous())
        g_binned = p.grad_x(F, f[perm].contiguous())
        p.synchronize()
        p.set_tuning(io_order="caller")
        assert torch.equal(p.forward(F), a_caller)
    assert torch.equal(a_binned, a_caller[perm])
    assert torch.equal(g_binned[0], g_caller[0][perm]) and torch.equal(g_binned[1], g_caller[1][perm])
    rel = (torch.linalg.vector_norm(A_binned - A_caller) / torch.linalg.vector_norm(A_caller)).item()
    assert rel < (1e-6 if prec == "f32" else 1e-14)
