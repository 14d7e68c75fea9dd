"""Batches (nfft2d_batch_*): many transforms of uneven size, one launch per
stage, CUDA-graph replay.  Each transform of a batch must match the same
transform run alone on a plan (same kernels, same binning): rel-L2 <= 1e-6;
and the exact NDFT at the FP32 bar, rel-L2 <= 1e-5."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _problem(sizes, Ms, seed):
    rng = np.random.default_rng(seed)
    xs, Fs, fs = [], [], []
    for (n1, n2), m in zip(sizes, Ms):
        xs.append((rng.uniform(-0.5, 0.5, m).astype(np.float32), rng.uniform(-0.5, 0.5, m).astype(np.float32)))
        Fs.append((rng.standard_normal((n1, n2)) + 1j * rng.standard_normal((n1, n2))).astype(np.complex64))
        fs.append((rng.standard_normal(m) + 1j * rng.standard_normal(m)).astype(np.complex64))
    return xs, Fs, fs


def _single(n1, n2, x, F, f, K=6):
    from miscellaneous_gb300.nfft import Plan
    with Plan(n1, n2, K=K) as p:
        p.set_points(torch.from_numpy(x[0]).cuda(), torch.from_numpy(x[1]).cuda())
        a = p.forward(torch.from_numpy(F).cuda().reshape(-1))
        b = p.adjoint(torch.from_numpy(f).cuda())
        p.synchronize()
        return a.cpu().numpy(), b.cpu().numpy().reshape(-1)


@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_single_plans(orc, graph):
    from miscellaneous_gb300.nfft import Batch
    sizes = [(64, 64), (32, 48), (64, 64), (16, 16), (128, 64), (32, 48), (8, 8)]
    Ms = [3000, 1, 500, 0, 7000, 257, 40]
    with Batch(sizes, graph=graph) as bt:
        for call, seed in enumerate((1, 2)):  # second call: new inputs, same points (graph replay)
            xs, Fs, fs = _problem(sizes, Ms, 10)
            rng = np.random.default_rng(seed)
            Fs = [(rng.standard_normal(F.shape) + 1j * rng.standard_normal(F.shape)).astype(np.complex64) for F in Fs]
            if call == 0:
                bt.set_points([torch.from_numpy(x[0]).cuda() for x in xs], [torch.from_numpy(x[1]).cuda() for x in xs])
            outs = bt.forward([torch.from_numpy(F).cuda().reshape(-1) for F in Fs])
            adjs = bt.adjoint([torch.from_numpy(f).cuda() for f in fs])
            bt.synchronize()
            for t, ((n1, n2), x, F, f) in enumerate(zip(sizes, xs, Fs, fs)):
                a, b = _single(n1, n2, x, F, f)
                got_f, got_F = outs[t].cpu().numpy(), adjs[t].cpu().numpy()
                if Ms[t] == 0:
                    assert got_f.size == 0 and np.all(got_F == 0)
                    continue
                assert orc.rel_l2(got_f, a) < 1e-6, (call, t)
                assert orc.rel_l2(got_F, b) < 1e-6, (call, t)
                g1, g2 = x[0].astype(np.float64) * n1, x[1].astype(np.float64) * n2
                assert orc.rel_l2(got_f, orc.ndft_type2(F, g1, g2, sign=-1)) < 1e-5, (call, t)
                # the batched adjoint against the exact FP64 type-1 sum itself
                exact_F = orc.ndft_type1(f.astype(np.complex128), g1, g2, n1, n2, sign=+1)
                assert orc.rel_l2(got_F.reshape(n1, n2), exact_F) < 1e-5, (call, t)


def test_batch_rebinning_recaptures_the_graph(orc):
    from miscellaneous_gb300.nfft import Batch
    sizes = [(32, 32), (64, 32)]
    with Batch(sizes) as bt:
        for seed, Ms in ((3, [100, 900]), (4, [2000, 50])):
            xs, Fs, fs = _problem(sizes, Ms, seed)
            bt.set_points([torch.from_numpy(x[0]).cuda() for x in xs], [torch.from_numpy(x[1]).cuda() for x in xs])
            outs = bt.forward([torch.from_numpy(F).cuda().reshape(-1) for F in Fs])
            bt.synchronize()
            for t, ((n1, n2), x, F) in enumerate(zip(sizes, xs, Fs)):
                g1, g2 = x[0].astype(np.float64) * n1, x[1].astype(np.float64) * n2
                assert orc.rel_l2(outs[t].cpu().numpy(), orc.ndft_type2(F, g1, g2, sign=-1)) < 1e-5


def test_pso_shaped_batch_matches_single_plans(orc):
    """The PSO synthesis shape: 250 transforms of 1936 points on a 44 x 44
    grid (a grid that is not a whole number of 16 x 16 tiles), replayed twice
    from the captured graph."""
    from miscellaneous_gb300.nfft import Batch
    sizes = [(44, 44)] * 250
    Ms = [44 * 44] * 250
    xs, Fs, fs = _problem(sizes, Ms, seed=250)
    b = Batch(sizes)
    b.set_points([torch.from_numpy(x[0]).cuda() for x in xs], [torch.from_numpy(x[1]).cuda() for x in xs])
    Ft = [torch.from_numpy(F).cuda().reshape(-1) for F in Fs]
    ft = [torch.from_numpy(f).cuda() for f in fs]
    for _ in range(2):
        outs_f = b.forward(Ft)
        outs_F = b.adjoint(ft)
        outs_R = b.spread_ref(ft)   # the reference's own sign, as its PSO code calls it
        b.synchronize()
    from miscellaneous_gb300.nfft import Plan
    for t in (0, 1, 77, 249):
        a, c = _single(44, 44, xs[t], Fs[t], fs[t])
        of, oF = outs_f[t].cpu().numpy(), outs_F[t].cpu().numpy().reshape(-1)
        assert np.linalg.norm(of - a) / np.linalg.norm(a) < 1e-6
        assert np.linalg.norm(oF - c) / np.linalg.norm(c) < 1e-6
        with Plan(44, 44) as p:
            p.set_points(torch.from_numpy(xs[t][0]).cuda(), torch.from_numpy(xs[t][1]).cuda())
            r = p.spread_ref(torch.from_numpy(fs[t]).cuda()).reshape(-1).cpu().numpy()
        oR = outs_R[t].cpu().numpy().reshape(-1)
        assert np.linalg.norm(oR - r) / np.linalg.norm(r) < 1e-6
        # the batched spread_ref and adjoint against the exact FP64 type-1 sums
        g1, g2 = xs[t][0].astype(np.float64) * 44, xs[t][1].astype(np.float64) * 44
        f64 = fs[t].astype(np.complex128)
        ex_R = orc.ndft_type1(f64, g1, g2, 44, 44, sign=-1).reshape(-1)
        ex_A = orc.ndft_type1(f64, g1, g2, 44, 44, sign=+1).reshape(-1)
        assert np.linalg.norm(oR - ex_R) / np.linalg.norm(ex_R) < 1e-5
        assert np.linalg.norm(oF - ex_A) / np.linalg.norm(ex_A) < 1e-5
    b.close()


@pytest.mark.parametrize("graph", [True, False])
def test_uneven_window_widths_in_one_batch(orc, graph):
    """A K per transform (nfft2d_batch_create_k): transforms in an order that
    interleaves the widths, including an empty one; each matches its own
    single plan of the same K, and the exact NDFT at the FP32 bar."""
    from miscellaneous_gb300.nfft import Batch
    sizes = [(64, 64), (32, 48), (64, 64), (16, 16), (128, 64), (32, 48), (48, 32), (64, 32)]
    Ks = [6, 3, 8, 4, 2, 6, 5, 7]
    Ms = [3000, 700, 2500, 0, 6000, 257, 900, 1500]
    xs, Fs, fs = _problem(sizes, Ms, 31)
    with Batch(sizes, K=Ks, graph=graph) as bt:
        bt.set_points([torch.from_numpy(x[0]).cuda() for x in xs], [torch.from_numpy(x[1]).cuda() for x in xs])
        outs = bt.forward([torch.from_numpy(F).cuda().reshape(-1) for F in Fs])
        adjs = bt.adjoint([torch.from_numpy(f).cuda() for f in fs])
        bt.synchronize()
        for t, ((n1, n2), K, x, F, f) in enumerate(zip(sizes, Ks, xs, Fs, fs)):
            got_f, got_F = outs[t].cpu().numpy(), adjs[t].cpu().numpy()
            if Ms[t] == 0:
                assert got_f.size == 0 and np.all(got_F == 0)
                continue
            a, b = _single(n1, n2, x, F, f, K=K)
            assert orc.rel_l2(got_f, a) < 1e-6, t
            assert orc.rel_l2(got_F, b) < 1e-6, t
            g1, g2 = x[0].astype(np.float64) * n1, x[1].astype(np.float64) * n2
            bar = 1e-5 if K >= 3 else 1e-3  # the window itself is off by 4e-4 at K = 2 (sigma = 2)
            assert orc.rel_l2(got_f, orc.ndft_type2(F, g1, g2, sign=-1)) < bar, t
            exact_F = orc.ndft_type1(f.astype(np.complex128), g1, g2, n1, n2, sign=+1)
            assert orc.rel_l2(got_F.reshape(n1, n2), exact_F) < bar, t


def test_batch_binning_reports_nonfinite_then_recovers(orc):
    """The batched binning (one CTA per transform) reports a NaN coordinate as
    NFFT2D_ERR_NONFINITE, like nfft2d_set_points, and the batch bins
    correctly afterwards."""
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.nfft import Batch
    sizes = [(32, 32), (48, 32), (32, 32)]
    Ms = [500, 700, 300]
    xs, Fs, _ = _problem(sizes, Ms, 21)
    bad = [(x[0].copy(), x[1].copy()) for x in xs]
    bad[1][0][17] = np.nan
    with Batch(sizes) as bt:
        with pytest.raises(_lib.NFFT2DError) as e:
            bt.set_points([torch.from_numpy(x[0]).cuda() for x in bad], [torch.from_numpy(x[1]).cuda() for x in bad])
        assert e.value.status == _lib.ERR_NONFINITE
        bt.set_points([torch.from_numpy(x[0]).cuda() for x in xs], [torch.from_numpy(x[1]).cuda() for x in xs])
        outs = bt.forward([torch.from_numpy(F).cuda().reshape(-1) for F in Fs])
        bt.synchronize()
        for t, ((n1, n2), x, F) in enumerate(zip(sizes, xs, Fs)):
            g1, g2 = x[0].astype(np.float64) * n1, x[1].astype(np.float64) * n2
            assert orc.rel_l2(outs[t].cpu().numpy(), orc.ndft_type2(F, g1, g2, sign=-1)) < 1e-5, t
