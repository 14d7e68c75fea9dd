"""Differentiation of the forward (type-2) transform.

* nfft2d_grad_x against the NDFT-derived exact gradient (oracle) and the
  restated-algorithm gradient (window-derivative gather);
* central finite differences (h = 1e-4, FP64 plan) of
  L = ||NFFT(f; x) - y||^2 at N = 32 x 32, M = 1024 (the least-squares case);
* a torch.autograd.Function wrapper, defined HERE in the test harness only,
  checked with torch.autograd.gradcheck.
Tolerances are written per assertion."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _setup(N=32, M=1024, seed=0, prec="f64"):
    rng = np.random.default_rng(seed)
    F = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    x1 = rng.uniform(-0.5, 0.5, M)
    x2 = rng.uniform(-0.5, 0.5, M)
    if prec == "f32":
        x1, x2 = x1.astype(np.float32), x2.astype(np.float32)
    v = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    return F, x1, x2, v


def _grad(F, x1, x2, v, prec, K=6, units="unit"):
    from miscellaneous_gb300.nfft import Plan
    N1, N2 = F.shape
    cdt = torch.complex64 if prec == "f32" else torch.complex128
    with Plan(N1, N2, K=K, precision=prec) as p:
        p.set_points(torch.from_numpy(x1).cuda(), torch.from_numpy(x2).cuda(), units=units)
        g1, g2 = p.grad_x(torch.from_numpy(F).to(cdt).cuda(), torch.from_numpy(v).to(cdt).cuda())
        p.synchronize()
    return g1.cpu().numpy().astype(np.float64), g2.cpu().numpy().astype(np.float64)


def _exact(orc, F, x1, x2, v):
    N1, N2 = F.shape
    d1, d2 = orc.ndft_type2_grad(F, x1.astype(np.float64) * N1, x2.astype(np.float64) * N2, sign=-1)
    # unit coordinates: d/dx_unit = N * d/dx_grid ; contracted with conj(v)
    return (np.real(np.conj(v) * d1) * N1, np.real(np.conj(v) * d2) * N2)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("prec,tol", [("f64", 1e-9), ("f32", 2e-5)])
def test_grad_x_vs_ndft_gradient(orc, prec, tol):
    F, x1, x2, v = _setup(prec=prec)
    g1, g2 = _grad(F, x1, x2, v, prec)
    e1, e2 = _exact(orc, F, x1, x2, v)
    assert _rel(g1, e1) < tol and _rel(g2, e2) < tol


def test_grad_x_f64_vs_restated_algorithm(orc):
    F, x1, x2, v = _setup(N=24, M=500, seed=2)
    g1, g2 = _grad(F, x1, x2, v, "f64")
    a1, a2 = orc.nfft1_2d_grad(F, x1 * 24, x2 * 24, sign=-1)
    assert _rel(g1, np.real(np.conj(v) * a1) * 24) < 1e-11
    assert _rel(g2, np.real(np.conj(v) * a2) * 24) < 1e-11


def test_grad_x_tiled_and_direct_f32_agree():
    from miscellaneous_gb300.nfft import Plan
    F, x1, x2, v = _setup(N=64, M=3000, seed=3, prec="f32")
    res = []
    for variant in (1, 2):
        with Plan(64, 64) as p:
            p.set_tuning(gather_variant=variant)
            p.set_points(torch.from_numpy(x1).cuda(), torch.from_numpy(x2).cuda())
            g = p.grad_x(torch.from_numpy(F).to(torch.complex64).cuda(), torch.from_numpy(v).to(torch.complex64).cuda())
            p.synchronize()
            res.append([t.cpu().numpy() for t in g])
    assert _rel(res[0][0], res[1][0]) < 1e-6 and _rel(res[0][1], res[1][1]) < 1e-6


def test_least_squares_loss_finite_differences():
    """L(x) = ||A(F; x) - y||^2 at N = 32^2, M = 1024; dL/dx vs central FD, h = 1e-4.
    Central differences carry a truncation error ~ (2 pi k_max h)^2 / 6 ~ 2e-5
    (k_max = 16) relative to the scale of the terms 2 Re(conj(r) df/dx), which
    cancel to much smaller values at some points; the tolerance is therefore
    2e-4 times the largest gradient component."""
    from miscellaneous_gb300.nfft import Plan
    rng = np.random.default_rng(5)
    N, M, h = 32, 1024, 1e-4
    F = torch.from_numpy(rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).cuda()
    x1 = torch.from_numpy(rng.uniform(-0.5, 0.5, M)).cuda()
    x2 = torch.from_numpy(rng.uniform(-0.5, 0.5, M)).cuda()
    y = torch.from_numpy(rng.standard_normal(M) + 1j * rng.standard_normal(M)).cuda()
    with Plan(N, N, precision="f64") as p:
        def loss(a, b):
            p.set_points(a, b)
            return float(torch.sum(torch.abs(p.forward(F) - y) ** 2))
        p.set_points(x1, x2)
        r = p.forward(F) - y
        g1, g2 = p.grad_x(F, 2 * r)
        scale = float(torch.max(torch.maximum(g1.abs(), g2.abs())))
        idx = rng.choice(M, 16, replace=False)
        for i in idx:
            e = torch.zeros(M, dtype=torch.float64, device="cuda")
            e[i] = h
            fd1 = (loss(x1 + e, x2) - loss(x1 - e, x2)) / (2 * h)
            fd2 = (loss(x1, x2 + e) - loss(x1, x2 - e)) / (2 * h)
            assert abs(fd1 - g1[i].item()) < 2e-4 * scale
            assert abs(fd2 - g2[i].item()) < 2e-4 * scale


class _NFFTForward(torch.autograd.Function):
    """Test-harness autograd wrapper: f = NFFT(F; x1, x2), FP64 plan.
    dL/dF = adjoint(grad_f); dL/dx = Re(conj(grad_f) df/dx) via grad_x."""

    @staticmethod
    def forward(ctx, F, x1, x2, plan):
        plan.set_points(x1.detach().contiguous(), x2.detach().contiguous())
        f = plan.forward(F.detach().contiguous().reshape(-1))
        ctx.save_for_backward(F, x1, x2)
        ctx.plan = plan
        return f

    @staticmethod
    def backward(ctx, gf):
        F, x1, x2 = ctx.saved_tensors
        p = ctx.plan
        p.set_points(x1.detach().contiguous(), x2.detach().contiguous())
        gf = gf.contiguous()
        gF = p.adjoint(gf).reshape(F.shape) if ctx.needs_input_grad[0] else None
        g1 = g2 = None
        if ctx.needs_input_grad[1] or ctx.needs_input_grad[2]:
            g1, g2 = p.grad_x(F.detach().contiguous().reshape(-1), gf)
        return gF, g1, g2, None


def test_autograd_function_gradcheck():
    from miscellaneous_gb300.nfft import Plan
    rng = np.random.default_rng(9)
    N, M = 8, 12
    F = torch.from_numpy(rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).cuda().requires_grad_()
    x1 = torch.from_numpy(rng.uniform(-0.45, 0.45, M)).cuda().requires_grad_()
    x2 = torch.from_numpy(rng.uniform(-0.45, 0.45, M)).cuda().requires_grad_()
    with Plan(N, N, K=6, precision="f64") as p:
        fn = lambda a, b, c: _NFFTForward.apply(a, b, c, p)  # noqa: E731
        assert torch.autograd.gradcheck(fn, (F, x1, x2), eps=1e-6, atol=1e-5, rtol=1e-4)
