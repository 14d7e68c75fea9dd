"""GPU parity of the Knab-window regridding (knabNFFT2D.m) against the CPU
oracle's restatement and the golden fixture of the independent numpy
transliteration; band-limited reproduction; extrapolation; plan reuse; the
one-call C entry point; error statuses."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "knab_golden.npz")

# FP32 path: rel-L2 <= 1e-5 against the FP64 oracle; FP64 path: the
# restatement's own NFFT1_2D error (c = 2, K = 6), ~1e-11
TOL = {"f32": 1e-5, "f64": 1e-10}


def _rel(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _run(dev, precision, ev, rho_in, cos_in, data, rho_out, cos_out, B1, B2, coord=None):
    import torch

    from miscellaneous_gb300 import knab
    cdt = torch.complex64 if precision == "f32" else torch.complex128
    rdt = coord or torch.float64
    r = knab.Regridder(rho_in, cos_in, B1, B2, precision=precision)
    r.set_points(torch.as_tensor(rho_out, dtype=rdt, device=dev).contiguous(),
                 torch.as_tensor(cos_out, dtype=rdt, device=dev).contiguous())
    out = r(torch.as_tensor(data, dtype=cdt, device=dev), ev)
    r.synchronize()
    info = r.info()
    r.close()
    return out.cpu().numpy(), info


def _geometry(seed, Nrows, Ncols, len1, len2, T1=0.3, T2=0.01, rot=0.04, margin=3):
    rng = np.random.default_rng(seed)
    rho_in = 100.0 + T1 * np.arange(Ncols)
    cos_in = -0.1 + T2 * np.arange(Nrows)
    r = np.linspace(rho_in[margin], rho_in[-1 - margin], len2)
    c = np.linspace(cos_in[margin], cos_in[-1 - margin], len1)
    Rg, Cg = np.meshgrid(r, c)
    u, v = (Rg - rho_in[0]) / T1, (Cg - cos_in[0]) / T2
    rho_out = rho_in[0] + T1 * (np.cos(rot) * u - 0.3 * np.sin(rot) * v)
    cos_out = cos_in[0] + T2 * (0.3 * np.sin(rot) * u + np.cos(rot) * v)
    data = rng.standard_normal((Nrows, Ncols)) + 1j * rng.standard_normal((Nrows, Ncols))
    return rho_in, cos_in, data, rho_out, cos_out


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_knab_golden(dev, precision):
    g = np.load(GOLDEN)
    out, info = _run(dev, precision, complex(g["extrap"]), g["rho_in"], g["cos_in"], g["data"], g["rho_out"],
                     g["cos_out"], float(g["B1"]), float(g["B2"]))
    assert (info["a"], info["b"], info["kgn"], info["kgm"]) == tuple(int(g[k]) for k in ("a", "b", "kgn", "kgm"))
    assert _rel(out, g["out"]) < TOL[precision]
    ev = complex(g["extrap"])
    assert np.all(out[:, 0] == np.complex128(ev).astype(out.dtype))
    assert np.all(out[-1, :] == np.complex128(ev).astype(out.dtype))


@pytest.mark.parametrize("precision", ["f32", "f64"])
@pytest.mark.parametrize("shape", [(48, 64, 40, 150), (64, 40, 170, 36), (30, 50, 29, 31)])
def test_knab_vs_oracle(dev, orc, precision, shape):
    # dense outputs along one axis give a = 3 or b = 3; sparse ones a = b = 2
    Nrows, Ncols, len1, len2 = shape
    rho_in, cos_in, data, rho_out, cos_out = _geometry(1, Nrows, Ncols, len1, len2)
    B1, B2 = 0.45 / 0.3, 0.4 / 0.01
    ref, rinfo = orc.knab_nfft2d(0.0, rho_in, cos_in, data, rho_out, cos_out, B1, B2)
    out, info = _run(dev, precision, 0.0, rho_in, cos_in, data, rho_out, cos_out, B1, B2)
    assert (info["a"], info["b"], info["kgn"], info["kgm"]) == (rinfo["a"], rinfo["b"], rinfo["kgn"], rinfo["kgm"])
    assert info["N1"] == info["b"] * Nrows and info["N2"] == info["a"] * Ncols
    assert _rel(out, ref) < TOL[precision]


def test_knab_float32_coordinates(dev, orc):
    import torch
    rho_in, cos_in, data, rho_out, cos_out = _geometry(2, 40, 48, 36, 60)
    # coordinates representable in FP32 so both sides see the same points
    rho_out = rho_out.astype(np.float32).astype(np.float64)
    cos_out = cos_out.astype(np.float32).astype(np.float64)
    B1, B2 = 0.45 / 0.3, 0.4 / 0.01
    ref, _ = orc.knab_nfft2d(0.0, rho_in, cos_in, data, rho_out, cos_out, B1, B2)
    out, _ = _run(dev, "f64", 0.0, rho_in, cos_in, data, rho_out, cos_out, B1, B2, coord=torch.float32)
    assert _rel(out, ref) < 1e-10


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_knab_reproduces_bandlimited_signal(dev, precision):
    Ncols, Nrows, T1, T2 = 128, 112, 0.3, 0.01
    rho_in = 100 + T1 * np.arange(Ncols)
    cos_in = -0.1 + T2 * np.arange(Nrows)
    tones = [(0.2 / T1, -0.15 / T2, 1.0), (-0.1 / T1, 0.2 / T2, 0.5 + 0.3j), (0.05 / T1, 0.05 / T2, -0.7j)]

    def s(r, c):
        return sum(a * np.exp(2j * np.pi * (f1 * (r - rho_in[0]) + f2 * (c - cos_in[0]))) for f1, f2, a in tones)
    R, C = np.meshgrid(rho_in, cos_in)
    RO, CO = np.meshgrid(np.linspace(rho_in[22], rho_in[-23], 250), np.linspace(cos_in[22], cos_in[-23], 68))
    out, _ = _run(dev, precision, np.nan, rho_in, cos_in, s(R, C), RO, CO, 0.5 / T1, 0.5 / T2)
    assert _rel(out, s(RO, CO)) < (2e-6 if precision == "f32" else 1e-10)


def test_knab_extrapolation_masks(dev, orc):
    rho_in, cos_in, data, rho_out, cos_out = _geometry(3, 32, 40, 24, 30)
    rho_out[:, 3] = rho_in[-1] + 0.01       # column 3 above the rho range (row 0 decides)
    rho_out[5, 7] = rho_in[0] - 5.0         # not row 0: no mask
    cos_out[10, :] = cos_in[0] - 0.001      # row 10 below the cos range (column 0 decides)
    cos_out[:, 0][[2, 4]] = cos_in[-1] + 1  # rows 2 and 4 via column 0
    B1, B2 = 0.45 / 0.3, 0.4 / 0.01
    ev = -1.5 + 2.25j
    ref, _ = orc.knab_nfft2d(ev, rho_in, cos_in, data, rho_out, cos_out, B1, B2)
    out, info = _run(dev, "f64", ev, rho_in, cos_in, data, rho_out, cos_out, B1, B2)
    mask = np.zeros(out.shape, bool)
    mask[:, 3] = True
    mask[[2, 4, 10], :] = True
    assert np.all(out[mask] == ev) and np.all(ref[mask] == ev)
    assert not np.any(out[~mask] == ev)
    assert info["masked_lines"] == 4
    assert _rel(out[~mask], ref[~mask]) < 1e-10


def test_knab_plan_reuse_and_rebind(dev, orc):
    import torch

    from miscellaneous_gb300 import knab
    rho_in, cos_in, data, rho_out, cos_out = _geometry(4, 40, 48, 36, 60)
    data2 = np.random.default_rng(9).standard_normal(data.shape) + 0j
    B1, B2 = 0.45 / 0.3, 0.4 / 0.01
    r = knab.Regridder(rho_in, cos_in, B1, B2, precision="f64")
    r.set_points(torch.tensor(rho_out, device=dev), torch.tensor(cos_out, device=dev))
    a1 = r(torch.tensor(data, device=dev)).cpu().numpy()
    a2 = r(torch.tensor(data2, device=dev)).cpu().numpy()
    # denser outputs: a changes, the internal plan is rebuilt
    _, _, _, rho_o3, cos_o3 = _geometry(4, 40, 48, 36, 150)
    r.set_points(torch.tensor(rho_o3, device=dev), torch.tensor(cos_o3, device=dev))
    a3 = r(torch.tensor(data, device=dev)).cpu().numpy()
    info = r.info()
    r.close()
    for out, d, ro, co in ((a1, data, rho_out, cos_out), (a2, data2, rho_out, cos_out), (a3, data, rho_o3, cos_o3)):
        ref, _ = orc.knab_nfft2d(0.0, rho_in, cos_in, d, ro, co, B1, B2)
        assert _rel(out, ref) < 1e-10
    assert info["a"] == 4


def test_knab_one_call_entry_point_matches_regridder(dev, lib):
    import torch
    rho_in, cos_in, data, rho_out, cos_out = _geometry(5, 40, 48, 36, 60)
    B1, B2 = 0.45 / 0.3, 0.4 / 0.01
    ref, _ = _run(dev, "f32", 0.5, rho_in, cos_in, data, rho_out, cos_out, B1, B2)
    d = torch.tensor(data, dtype=torch.complex64, device=dev)
    ro = torch.tensor(rho_out, device=dev)
    co = torch.tensor(cos_out, device=dev)
    out = torch.empty(rho_out.shape, dtype=torch.complex64, device=dev)
    ri = np.ascontiguousarray(rho_in)
    ci = np.ascontiguousarray(cos_in)
    torch.cuda.synchronize()
    st = lib.nfft2d_knab_nfft2d(0.5, 0.0, ri.ctypes.data_as(ctypes.c_void_p), ri.size,
                                ci.ctypes.data_as(ctypes.c_void_p), ci.size, ctypes.c_void_p(d.data_ptr()),
                                ctypes.c_void_p(ro.data_ptr()), ctypes.c_void_p(co.data_ptr()), rho_out.shape[0],
                                rho_out.shape[1], B1, B2, 0, ctypes.c_void_p(out.data_ptr()),
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_knab_matlab_mirror_accepts_meshgrid_axes(dev, orc):
    import torch

    from miscellaneous_gb300 import knab
    rho_in, cos_in, data, rho_out, cos_out = _geometry(6, 24, 32, 20, 28)
    RHO_IN, COSALPHA_IN = np.meshgrid(rho_in, cos_in)
    B1, B2 = 0.45 / 0.3, 0.4 / 0.01
    out = knab.knabNFFT2D(0.0, RHO_IN, COSALPHA_IN, torch.tensor(data, device=dev), torch.tensor(rho_out, device=dev),
                          torch.tensor(cos_out, device=dev), B1, B2).cpu().numpy()
    ref, _ = orc.knab_nfft2d(0.0, rho_in, cos_in, data, rho_out, cos_out, B1, B2)
    assert _rel(out, ref) < 1e-10


def test_knab_error_statuses(dev):
    import torch

    from miscellaneous_gb300 import knab
    from miscellaneous_gb300._lib import ERR_INVALID_ARG, ERR_NONFINITE, NFFT2DError
    # an odd NFFT1_2D size: b = 3 with 21 rows -> N1 = 63, which the reference cannot run
    rho_in, cos_in, data, rho_out, cos_out = _geometry(7, 21, 32, 43, 20)
    r = knab.Regridder(rho_in, cos_in, 0.45 / 0.3, 0.4 / 0.01, precision="f32")
    with pytest.raises(NFFT2DError) as e:
        r.set_points(torch.tensor(rho_out, device=dev), torch.tensor(cos_out, device=dev))
    assert e.value.status == ERR_INVALID_ARG
    with pytest.raises(RuntimeError):
        r(torch.zeros(21, 32, dtype=torch.complex64, device=dev))
    # a NaN output coordinate is refused
    ro = np.ascontiguousarray(rho_out[:20])
    ro[3, 4] = np.nan
    with pytest.raises(NFFT2DError) as e:
        r.set_points(torch.tensor(ro, device=dev), torch.tensor(np.ascontiguousarray(cos_out[:20]), device=dev))
    assert e.value.status == ERR_NONFINITE
    r.close()
    with pytest.raises(NFFT2DError):
        knab.Regridder(rho_in, cos_in, 0.0, 1.0)            # B = 0
    with pytest.raises(NFFT2DError):
        knab.Regridder(rho_in[:1], cos_in, 1.0, 1.0)        # fewer than 2 columns
