"""World-size-2 gloo tests (CPU) of the sharding logic in
miscellaneous_gb300/shard.py.  The local transform on each rank is the CPU
oracle standing in for the GPU plan; the collective and the slicing are the
product code under test."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from miscellaneous_gb300.shard import shard_batch, shard_bounds


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _problem():
    rng = np.random.default_rng(11)
    N1, N2, M = 16, 12, 301
    F = rng.standard_normal((N1, N2)) + 1j * rng.standard_normal((N1, N2))
    x1 = (rng.random(M) - 0.5) * N1
    x2 = (rng.random(M) - 0.5) * N2
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    return N1, N2, M, F, x1, x2, f


def _worker(rank, world, port, outdir):
    import oracle
    from miscellaneous_gb300.shard import sharded_adjoint, sharded_forward
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    oracle.set_threads(1)
    N1, N2, M, F, x1, x2, f = _problem()
    s, e = shard_bounds(M, rank, world)

    def t1(fl):
        out = oracle.nfft2_2d(fl.numpy(), x1[s:e], x2[s:e], N1, N2, sign=+1)
        return torch.from_numpy(out)

    def t2(Fc):
        return torch.from_numpy(oracle.nfft1_2d(Fc.numpy(), x1[s:e], x2[s:e], sign=-1))

    Fa = sharded_adjoint(t1, torch.from_numpy(f[s:e]))
    fw = sharded_forward(t2, torch.from_numpy(F))
    np.save(os.path.join(outdir, f"adj{rank}.npy"), Fa.numpy())
    np.save(os.path.join(outdir, f"fwd{rank}.npy"), fw.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_shard_bounds_cover_exactly():
    for M in (0, 1, 7, 100, 1001):
        for world in (1, 2, 3, 8):
            spans = [shard_bounds(M, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == M
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [e - s for s, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)
    assert shard_batch(5, 1, 2) == [1, 3]


def test_two_rank_sharded_transforms_match_single_rank(orc, tmp_path):
    world = 2
    port = _free_port()
    mp.spawn(_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    N1, N2, M, F, x1, x2, f = _problem()
    full_adj = orc.nfft2_2d(f, x1, x2, N1, N2, sign=+1)
    full_fwd = orc.nfft1_2d(F, x1, x2, sign=-1)
    for r in range(world):
        assert orc.rel_l2(np.load(tmp_path / f"adj{r}.npy"), full_adj) < 1e-12
    fwd = np.concatenate([np.load(tmp_path / f"fwd{r}.npy") for r in range(world)])
    assert orc.rel_l2(fwd, full_fwd) < 1e-13
