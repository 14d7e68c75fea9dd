"""Benchmark of the 2D NFFT hot path on GB300.

Workload (default): the large clustered NFFT, the largest single-GPU
configuration -- N = 2048 x 2048 complex64 coefficients (re/im ~ N(0,1)),
M = 2^24 points with each coordinate ~ N(0, 0.15^2) wrapped into
[-0.5, 0.5); sigma = 2, w = K = 6 (13 x 13 taps), FP32 with compensated
gather accumulation and FP64 coordinate reduction and deapodization tables.
Seeded synthetic data (NumPy PCG64, seed 3).  The configuration is a
precision study: the line also carries the step time and the error of
w = 4 and w = 8 on the same points (precision_study).

One step = one forward (type 2, reference NFFT1_2D) + one adjoint (type 1,
sign +1) over the same points with the points already binned (the plan is
reused, as a solver iteration does).  value = points per second through one
forward+adjoint pair = M / step time.  The working set (about 700 MB) is
larger than L2, and a 256 MB buffer is written between timed steps (outside
the timed events) all the same.  The timed steps run without the plan's
per-stage events; the stage breakdown (stages_ms, and the roofline's kernel
time) comes from as many further steps with them.

e2e = the same metric through the public API with HOST (pinned) buffers:
each step copies x1, x2, F and f host->device, bins the points
(set_points, asynchronous), runs forward + adjoint and copies f_out and
F_out back; L2 is flushed between these steps too.

Other workloads (--workload): polar (the SAR polar raster, 512^2, 2^20
points), config1 (64^2, 4096 points), batch (64 uneven transforms), pso (250
transforms on 44^2), lsq (least-squares gradient step, 1024^2, 2^22 points),
knab (the Knab-window regridding of a 1024^2 raster onto 2048^2 outputs).
Every line reports rel-L2 against FP64 sums on a subset of the points.

--impl reference times the reference's CPU algorithm (the C restatement of
NFFT1_2D.m / NFFT2_2D.m in oracle/, OpenMP over all host cores) on the same
workload, and the reference's own GPU spreading (NFFT/NFFT2_2D.cu, built
into oracle/_ref) on two small shapes (reference_gpu_spread); the library's
line carries its own times on those shapes (spread_small_cases).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "NU points/s, 2D type-2 NFFT at rel-L2<=1e-5 vs FP64 NDFT; fwd+adjoint ms/iter"
UNIT = "points/s"
L2_BYTES = 129 << 20  # GB300 L2
L2_FLUSH_BYTES = 256 << 20


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def polar_raster(seed: int = 2, spokes: int = 512, samples: int = 2048, N: int = 512, jitter: float = 1e-3,
                 K: int = 6):
    rng = np.random.default_rng(seed)
    theta = np.pi * np.arange(spokes) / spokes
    r = -0.5 + np.arange(samples) / samples
    R, TH = np.meshgrid(r, theta, indexing="ij")
    x1 = (R * np.cos(TH)).ravel() + rng.uniform(-jitter, jitter, R.size)
    x2 = (R * np.sin(TH)).ravel() + rng.uniform(-jitter, jitter, R.size)
    x1 = np.mod(x1 + 0.5, 1.0) - 0.5
    x2 = np.mod(x2 + 0.5, 1.0) - 0.5
    F = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    f = (rng.standard_normal(x1.size) + 1j * rng.standard_normal(x1.size)).astype(np.complex64)
    return dict(name="polar_raster_512x512_1M" + ("" if K == 6 else f"_K{K}"), N1=N, N2=N, sigma=2.0, K=K,
                x1=x1.astype(np.float32), x2=x2.astype(np.float32), F=F, f=f,
                config={"workload": "polar-raster NFFT (SAR back-projection shape)", "N": [N, N],
                        "points": int(x1.size), "spokes": spokes, "samples_per_spoke": samples,
                        "jitter": jitter, "sigma": 2.0, "w": K, "taps": f"{2 * K + 1}x{2 * K + 1}", "seed": seed})


def uniform_config1(seed: int = 0):
    rng = np.random.default_rng(seed)
    N, M = 64, 4096
    F = (rng.uniform(-1, 1, (N, N)) + 1j * rng.uniform(-1, 1, (N, N))).astype(np.complex64)
    x1 = rng.uniform(-0.5, 0.5, M).astype(np.float32)
    x2 = rng.uniform(-0.5, 0.5, M).astype(np.float32)
    f = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    return dict(name="uniform_64x64_4096", N1=N, N2=N, sigma=2.0, K=6, x1=x1, x2=x2, F=F, f=f,
                config={"workload": "plain 2D NFFT vs NDFT2_2D", "N": [N, N], "points": M, "sigma": 2.0,
                        "w": 6, "seed": seed})


def clustered_config3(seed: int = 3, K: int = 6, M: int = 1 << 24, N: int = 2048):
    rng = np.random.default_rng(seed)
    x1 = np.mod(rng.normal(0.0, 0.15, M) + 0.5, 1.0) - 0.5
    x2 = np.mod(rng.normal(0.0, 0.15, M) + 0.5, 1.0) - 0.5
    F = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    f = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    return dict(name=f"clustered_{N}x{N}_{M}_K{K}", N1=N, N2=N, sigma=2.0, K=K,
                x1=x1.astype(np.float32), x2=x2.astype(np.float32), F=F, f=f,
                config={"workload": "large clustered NFFT", "N": [N, N], "points": M, "sigma": 2.0, "w": K,
                        "seed": seed})


def least_squares_config5(seed: int = 5, N: int = 1024, M: int = 1 << 22, noise: float = 1e-3):
    """L(f, x) = ||NFFT(f; x) - y||^2 with y = NFFT(f_true; x) + CN(0, noise^2):
    N = 1024^2, M = 2^22 uniform points, sigma 2, w 6 (y is built on the GPU)."""
    rng = np.random.default_rng(seed)
    x1 = rng.uniform(-0.5, 0.5, M).astype(np.float32)
    x2 = rng.uniform(-0.5, 0.5, M).astype(np.float32)
    f_true = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    F0 = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    e = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64) * np.float32(noise / np.sqrt(2))
    return dict(name=f"least_squares_{N}x{N}_{M}", N1=N, N2=N, sigma=2.0, K=6, x1=x1, x2=x2, F=F0, f_true=f_true,
                noise=e, config={"workload": "differentiable least-squares NFFT", "N": [N, N], "points": M,
                                 "sigma": 2.0, "w": 6, "noise": noise, "seed": seed})


def knab_regrid(seed: int = 5, N: int = 1024, L: int = 2048):
    """Knab-window regridding (knabNFFT2D.m), the FFBP sub-image step: an
    N x N raster on a (cos alpha, rho) grid -- range spacing 0.15, angle
    spacing 1/N, bandwidths 0.5/T as FBP.m:95 passes them -- regridded to an
    L x L output raster covering the input's interior, rotated slightly so
    the output points are not separable."""
    rng = np.random.default_rng(seed)
    T1, T2 = 0.15, 1.0 / N
    rho_in = 1000.0 + T1 * np.arange(N)
    cos_in = -0.5 + T2 * np.arange(N)
    m = 24  # stay P = 18 samples away from the raster's edges
    r = np.linspace(rho_in[m], rho_in[-1 - m], L)
    c = np.linspace(cos_in[m], cos_in[-1 - m], L)
    Rg, Cg = np.meshgrid(r, c)
    u, v = (Rg - rho_in[0]) / T1, (Cg - cos_in[0]) / T2
    th = 0.01
    rho_out = rho_in[0] + T1 * (np.cos(th) * u - np.sin(th) * v)
    cos_out = cos_in[0] + T2 * (np.sin(th) * u + np.cos(th) * v)
    data = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    return dict(name=f"knab_{N}x{N}_to_{L}x{L}", rho_in=rho_in, cos_in=cos_in, rho_out=rho_out, cos_out=cos_out,
                data=data, B1=0.5 / T1, B2=0.5 / T2,
                config={"workload": "Knab-window regridding (knabNFFT2D)", "raster": [N, N], "outputs": [L, L],
                        "P": 18, "sigma": 2.0, "w": 6, "bandwidth": "0.5/T", "seed": seed})


def uneven_batch(seed: int = 4, count: int = 64):
    """64 transforms, N = 2^e with e ~ U{7..10} (square), M log-uniform in
    [1e4, 4e6], points uniform, coefficients N(0,1) complex; sigma 2, w 6."""
    rng = np.random.default_rng(seed)
    es = rng.integers(7, 11, count)
    Ms = np.floor(10 ** rng.uniform(4, np.log10(4e6), count)).astype(np.int64)
    items = []
    for e, m in zip(es, Ms):
        N = 1 << int(e)
        items.append(dict(N=N, M=int(m)))
    return dict(name="uneven_batch_64", items=items, seed=seed, sigma=2.0, K=6,
                config={"workload": "uneven batch of 64 transforms", "count": count, "N": "2^U{7..10} square",
                        "points": int(Ms.sum()), "points_per_transform": "floor(10^U(4, log10 4e6))", "sigma": 2.0,
                        "w": 6, "seed": seed})


def pso_batch(seed: int = 6, count: int = 250):
    """The reflectarray PSO synthesis' far-field step for one generation
    (Synthesis/PSO/Synthesis.cu:385-405 for each of the 250 particles of
    PSO.cu:27): 44 x 44 elements at 14.25 GHz (kernel_single_v2.cu:23-31),
    spectral oversampling chi' = 4 (:72-80), so Nu = Nv = 44 and each far
    field is 88 x 88; element positions on a 0.6-wavelength lattice with a
    seeded +-0.05-wavelength jitter per particle (aperiodic arrays), unit
    excitations with seeded phases, the visible-region filter.  One step =
    the scaling, binning, reference-sign spread and filter for every
    particle (positions change every generation, so the binning is in)."""
    rng = np.random.default_rng(seed)
    lam = 3e8 / 14.25e9
    Mx = My = 44
    aap = (Mx - 1) * (lam * 0.5 / 2.0)
    a_prime = 4 * aap
    beta = 2 * math.pi / lam
    Nu = int((beta / 2) / (math.pi / a_prime)) + 1
    Nv = int((beta / 2) / (math.pi / a_prime)) + 1
    a_prime_f = float(np.float32(a_prime))
    f32 = np.float32
    sx = float(f32(float(f32(2 * Nu * (math.pi / a_prime_f))) / (2.0 * math.pi)))
    sy = float(f32(float(f32(2 * Nv * (math.pi / a_prime_f))) / (2.0 * math.pi)))
    gx, gy = np.meshgrid((np.arange(Mx) - (Mx - 1) / 2) * 0.6 * lam, (np.arange(My) - (My - 1) / 2) * 0.6 * lam)
    X = [(gx + rng.uniform(-0.05, 0.05, gx.shape) * lam).ravel().astype(np.float32) for _ in range(count)]
    Y = [(gy + rng.uniform(-0.05, 0.05, gy.shape) * lam).ravel().astype(np.float32) for _ in range(count)]
    E = [np.exp(1j * rng.uniform(-math.pi, math.pi, gx.size)).astype(np.complex64) for _ in range(count)]
    u = np.arange(-Nu, Nu) * (math.pi / a_prime)
    v = np.arange(-Nv, Nv) * (math.pi / a_prime)
    V, U = np.meshgrid(v, u, indexing="ij")
    filt = (U * U + V * V <= beta * beta).astype(np.float32)
    return dict(name=f"pso_far_field_{count}x{2 * Nv}x{2 * Nu}_{Mx * My}", X=X, Y=Y, E=E, Nu=Nu, Nv=Nv, sx=sx, sy=sy,
                filter=filt, count=count, M=Mx * My,
                config={"workload": "PSO reflectarray far field, one generation (scaling + binning + NFFT2_2D_GPU "
                                    "sign + filter per particle)", "particles": count, "far_field": [2 * Nv, 2 * Nu],
                        "elements": [Mx, My], "points": count * Mx * My, "sigma": 2.0, "w": 6, "seed": seed})


def run_pso(args, wl):
    """One generation's far fields: the batched step (nfft2d_batch_far_field)
    vs one plan per particle (set_points + spread_ref + filter, the shape of
    the reference's per-particle loop, through the library)."""
    import torch

    from miscellaneous_gb300.nfft import Batch, Plan
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    n1, n2, P, M = 2 * wl["Nv"], 2 * wl["Nu"], wl["count"], wl["M"]
    X = [torch.from_numpy(a).to(dev) for a in wl["X"]]
    Y = [torch.from_numpy(a).to(dev) for a in wl["Y"]]
    E = [torch.from_numpy(a).to(dev) for a in wl["E"]]
    filt = torch.from_numpy(wl["filter"].ravel()).to(dev)
    outs = [torch.empty(n1 * n2, dtype=torch.complex64, device=dev) for _ in range(P)]
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    batch = Batch([(n1, n2)] * P, sigma=2.0, K=6, stream=stream)

    def batched():
        batch.far_field(X, Y, E, wl["sx"], wl["sy"], filt, outs)

    plans = [Plan(n1, n2, sigma=2.0, K=6, stream=stream) for _ in range(P)]
    xs = [torch.empty(M, dtype=torch.float32, device=dev) for _ in range(P)]
    ys = [torch.empty(M, dtype=torch.float32, device=dev) for _ in range(P)]

    def sequential():
        for p in range(P):
            torch.mul(X[p], wl["sx"], out=xs[p])
            torch.mul(Y[p], wl["sy"], out=ys[p])
            plans[p].set_points(xs[p], ys[p], units="grid")
            plans[p].spread_ref(E[p], out=outs[p])
            outs[p].mul_(filt)

    def timed(step):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            ev0.record(stream)
            step()
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
        return statistics.median(ms)

    with ClockSampler(0) as clocks:
        t_batch = timed(batched)
    t_seq = timed(sequential)
    batched()
    batch.synchronize()
    # accuracy: a few particles against the exact FP64 type-1 sum at the FP32-scaled points
    errs = []
    for p in (0, P // 2, P - 1):
        x1 = (X[p] * wl["sx"]).double() / n1
        x2 = (Y[p] * wl["sy"]).double() / n2
        ref = ndft_type1(E[p], x1, x2, n1, n2, -1, torch) * filt.reshape(n1, n2)
        errs.append(rel_l2(outs[p], ref, torch))
    total = P * M
    line = {"metric": METRIC, "value": total / (t_batch * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_batch, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": wl["config"],
            "sequential_ms_per_step": t_seq, "batched_speedup": t_seq / t_batch,
            "sequential": "one library plan per particle: set_points + spread_ref + filter, as the reference's loop",
            "batched": "nfft2d_batch_far_field: FP32 scaling, binning, reference-sign spread and filter for all "
                       "particles",
            "accuracy": {"rel_l2_max": max(errs), "particles_checked": 3,
                         "oracle": "exact FP64 type-1 sum at the FP32-scaled points, times the filter"},
            "clocks": clocks.summary()}
    print(json.dumps(line))
    for p in plans:
        p.close()
    batch.close()


def run_pso_reference(args, wl):
    """The reference's own far-field loop on the GPU: one NFFT2_2D_GPU call
    (NFFT/NFFT2_2D.cu compiled unchanged into oracle/_ref, dynamic-parallelism
    interpolation) per particle, with the FP32 scaling and the filter around
    it, for the same generation."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import torch

    from oracle import ref_gpu
    if not torch.cuda.is_available() or not ref_gpu.available():
        print(json.dumps({"impl": "reference", "unavailable": "the reference's NFFT2_2D_GPU needs a GPU and "
                                                              "oracle/_ref/nfft2_2d_ref.cubin"}))
        return
    dev = torch.device("cuda", 0)
    n1, n2, P, M = 2 * wl["Nv"], 2 * wl["Nu"], wl["count"], wl["M"]
    X = [torch.from_numpy(a).to(dev) for a in wl["X"]]
    Y = [torch.from_numpy(a).to(dev) for a in wl["Y"]]
    E = [torch.from_numpy(a).to(dev) for a in wl["E"]]
    filt = torch.from_numpy(wl["filter"]).to(dev)
    steps = min(args.steps, 3)

    def generation():
        for p in range(P):
            ff = ref_gpu.nfft2_2d_gpu(E[p], X[p] * wl["sx"], Y[p] * wl["sy"], n1, n2)
            ff.mul_(filt)
        torch.cuda.synchronize()

    generation()
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        generation()
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    value = P * M / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": 1, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": wl["config"],
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 0, "kind": "reference",
                             "sample": "the whole generation; the reference's own GPU code (NFFT/NFFT2_2D.cu, "
                                       "oracle/_ref) once per particle -- the reference has no CPU path for this "
                                       "step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def ffbp_scene(seed: int = 7, Np: int = 64, nf: int = 216, Nx: int = 128, step: float = 0.08, R: float = 10e3):
    """The reference's SAR scenario (BP_FBP_FFBP_main.m:7-103): a straight
    track at R = 10 km and 30 degrees depression, a 3-degree aperture,
    216 frequency samples over 600 MHz at 10 GHz, a 128 x 128 scene at 8 cm
    -- with 64 pulses instead of 128 (the 128-pulse recursion asks its Knab
    regridding for an odd NFFT grid that the reference's NFFT1_2D cannot take).
    Three unit point targets at seeded positions in the scene."""
    rng = np.random.default_rng(seed)
    c, fc, BW = 299792458.0, 10e9, 600e6
    deltaF = BW / nf
    minF = fc - BW / 2.0
    f2 = minF + nf * deltaF
    maxAz, dep = 3 * math.pi / 180, math.pi / 6
    az = np.arange(Np) / Np * maxAz - maxAz / 2
    X = R * math.cos(dep) * np.ones(Np)
    Y = R * math.cos(dep) * np.tan(az)
    Z = R * math.sin(dep) * np.ones(Np)
    R0 = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    W = Nx * step
    v = np.linspace(-W / 2, W / 2, Nx)
    x_mat, y_mat = np.meshgrid(v, v)
    targets = [(0.0, 0.0)] + [tuple(t) for t in rng.uniform(-0.4 * W, 0.4 * W, (2, 2))]
    fk = minF + np.arange(nf) * deltaF
    ph = np.zeros((nf, Np), dtype=np.complex128)
    for tx, ty in targets:
        dR = np.sqrt((X - tx) ** 2 + (Y - ty) ** 2 + Z ** 2) - R0
        ph += np.exp(-1j * 4 * math.pi * np.outer(fk, dR) / c)
    data = dict(AntX=X, AntY=Y, AntZ=Z, R0=R0, phdata=ph, x_mat=x_mat, y_mat=y_mat, z_mat=np.zeros_like(x_mat))
    return dict(name=f"ffbp_{Np}pulses_{nf}f_{Nx}x{Nx}", data=data, sar=dict(c=c, fc=fc, BW=BW, f2=f2), Np=Np,
                config={"workload": "FFBP SAR image formation (knabNFFT2D regridding, NFFT1_1D leaves)",
                        "pulses": Np, "frequency_samples": nf, "scene": [Nx, Nx], "pixel_m": step, "range_m": R,
                        "targets": len(targets), "seed": seed})


def type3_scene(seed: int = 8, M: int = 1 << 20, N: int = 1 << 20, eps: float = 1e-6):
    """Type-3 2D NUFFT (NUFFT_2D_CPU's problem): M nonuniform points with
    x ~ U(-40, 25), y ~ N(0, 6^2) and complex N(0, 1) values, N nonuniform
    frequencies s ~ U(-3, 4), t ~ U(-2.5, 2.5) (seeded PCG64), accuracy eps."""
    rng = np.random.default_rng(seed)
    x, y = rng.uniform(-40.0, 25.0, M), rng.normal(0.0, 6.0, M)
    f = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    s, t = rng.uniform(-3.0, 4.0, N), rng.uniform(-2.5, 2.5, N)
    return dict(name=f"type3_{M}_{N}", x=x, y=y, f=f, s=s, t=t, eps=eps,
                config={"workload": "type-3 2D NUFFT (Gaussian gridding)", "points": M, "frequencies": N,
                        "eps": eps, "x": "U(-40, 25)", "y": "N(0, 6^2)", "s": "U(-3, 4)", "t": "U(-2.5, 2.5)",
                        "seed": seed})


WORKLOADS = {"polar": polar_raster, "config1": uniform_config1, "clustered": clustered_config3, "batch": uneven_batch,
             "lsq": least_squares_config5, "knab": knab_regrid, "pso": pso_batch, "ffbp": ffbp_scene,
             "type3": type3_scene}


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
STAGES_NOTE = {
    False: "pad, fft_fwd (cuFFT), halo_fill, gather | spread (incl. grid zeroing), fold, fft_adj (cuFFT), crop",
    True: "fused FFT passes: pad = deapodize/pad + band-column FFT, fft_fwd = row FFT + halo fill, halo_fill = 0; "
          "fold = halo fold + row FFT, fft_adj = band-column FFT + crop, crop = 0; gather; spread (incl. grid zeroing)",
}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes of `kernel` on `workload` from the committed ncu
    summary (profiles/*.md lines 'traffic_bytes_per_launch[kernel@workload]: B')."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    pat = re.compile(r"traffic_bytes_per_launch\[" + re.escape(kernel) + "@" + re.escape(workload) +
                     r"\]:\s*([0-9.eE+]+)")
    for fn in sorted(os.listdir(pdir)):
        if not fn.endswith((".md", ".txt")):
            continue
        with open(os.path.join(pdir, fn)) as fh:
            m = pat.search(fh.read())
        if m:
            return float(m.group(1))
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.lines:
            return None
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---------------------------------------------------------------------------
# accuracy (FP64 NDFT on the GPU through torch complex128 GEMMs: a checker,
# independent of the product kernels)
# ---------------------------------------------------------------------------
def _phases(xg, N, sign, torch):
    k = torch.arange(N, device=xg.device, dtype=torch.float64) - N // 2
    a = xg[:, None] * k[None, :] / N
    a = a - torch.round(a)
    return torch.exp(1j * (2 * math.pi * sign) * a)


def ndft_type2_subset(F, x1, x2, idx, sign, torch):
    N1, N2 = F.shape
    xg1 = x1[idx].double() * N1
    xg2 = x2[idx].double() * N2
    out = torch.empty(idx.numel(), dtype=torch.complex128, device=F.device)
    Fd = F.to(torch.complex128)
    for s in range(0, idx.numel(), 8192):
        e1 = _phases(xg1[s:s + 8192], N1, sign, torch)
        e2 = _phases(xg2[s:s + 8192], N2, sign, torch)
        G = e2 @ Fd.T                     # (P, N1): sum_k2 F[k1, k2] e2[p, k2]
        out[s:s + 8192] = (G * e1).sum(1)
    return out


def ndft_type1(f, x1, x2, N1, N2, sign, torch):
    xg1 = x1.double() * N1
    xg2 = x2.double() * N2
    acc = torch.zeros(N1, N2, dtype=torch.complex128, device=f.device)
    fd = f.to(torch.complex128)
    for s in range(0, f.numel(), 16384):
        e1 = _phases(xg1[s:s + 16384], N1, sign, torch) * fd[s:s + 16384, None]
        e2 = _phases(xg2[s:s + 16384], N2, sign, torch)
        acc += e1.T @ e2
    return acc


def rel_l2(a, b, torch):
    a = a.reshape(-1).to(torch.complex128)
    b = b.reshape(-1).to(torch.complex128)
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


def subset_accuracy(f_fwd, F, f, x1, x2, N1, N2, nsub, seed, plan_kw, stream, torch):
    """Rel-L2 of a forward result f_fwd (all points) against the FP64 NDFT on
    a random subset of the points, and of the adjoint of f over that subset
    (a plan on the subset) against the FP64 type-1 sum."""
    from miscellaneous_gb300.nfft import Plan
    M = x1.numel()
    g = torch.Generator(device="cpu").manual_seed(seed)
    idx = torch.randperm(M, generator=g)[:min(M, nsub)].to(x1.device)
    e_fwd = rel_l2(f_fwd[idx], ndft_type2_subset(F.reshape(N1, N2), x1, x2, idx, -1, torch), torch)
    sub_plan = Plan(N1, N2, precision="f32", stream=stream, **plan_kw)
    sub_plan.set_points(x1[idx].contiguous(), x2[idx].contiguous(), units="unit")
    fa = sub_plan.adjoint(f[idx].contiguous())
    sub_plan.synchronize()
    e_adj = rel_l2(fa, ndft_type1(f[idx], x1[idx], x2[idx], N1, N2, +1, torch), torch)
    sub_plan.close()
    return e_fwd, e_adj, int(idx.numel()), idx


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement of the reference algorithm)
# ---------------------------------------------------------------------------
def cpu_reference_step(wl, idx):
    import oracle
    N1, N2 = wl["N1"], wl["N2"]
    g1 = wl["x1"][idx].astype(np.float64) * N1
    g2 = wl["x2"][idx].astype(np.float64) * N2
    t0 = time.perf_counter()
    oracle.nfft1_2d(wl["F"], g1, g2, c=wl["sigma"], K=wl["K"], sign=-1)
    oracle.nfft2_2d(wl["f"][idx], g1, g2, N1, N2, c=wl["sigma"], K=wl["K"], sign=+1)
    return time.perf_counter() - t0


def _cpu_sample(wl, rng, m):
    M = wl["x1"].size
    return np.sort(rng.choice(M, m, replace=False)) if m < M else np.arange(M)


def choose_cpu_sample(wl, max_step_s: float = 1.0):
    """Grow the point sample from 2^16 by 4x while one forward+adjoint step of
    the CPU restatement stays under max_step_s (the grid is always full)."""
    M = wl["x1"].size
    rng = np.random.default_rng(123)
    m = min(M, 1 << 16)
    idx = _cpu_sample(wl, rng, m)
    dt = cpu_reference_step(wl, idx)
    while m < M and dt * 4 < max_step_s:
        m = min(M, m * 4)
        idx = _cpu_sample(wl, rng, m)
        dt = cpu_reference_step(wl, idx)
    return idx, dt


def cpu_baseline_isolated(args, steps: int = 10):
    """The CPU baseline of the library's line, timed by the reference arm's
    own code (run_reference) in a child process that never creates a CUDA
    context: the restatement's per-step grids are large fresh allocations,
    and their page faults cost about twice as much in a process that holds
    a CUDA context and pinned host buffers, which would make the two arms'
    CPU figures disagree.  Returns the child's cpu_baseline object."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--workload", args.workload,
           "--steps", str(steps), "--warmup", "3", "--no-reference-gpu"]
    if args.K:
        cmd += ["--K", str(args.K)]
    if getattr(args, "points", None):
        cmd += ["--points", str(args.points)]
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "LOCAL_WORLD_SIZE")}
    env["CUDA_VISIBLE_DEVICES"] = ""
    try:
        res = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600, check=True)
        line = json.loads(res.stdout.strip().splitlines()[-1])
    except (subprocess.SubprocessError, ValueError, IndexError) as e:
        return {"unavailable": f"CPU baseline child process failed: {type(e).__name__}"}
    cb = dict(line["cpu_baseline"])
    cb["ms_per_step"] = line["ms_per_step"]
    cb["process"] = "child process without a CUDA context (the reference arm's code, --steps %d)" % steps
    return cb


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------
def small_spread_cases():
    """The two shapes on which the reference's own GPU spreading
    (NFFT/NFFT2_2D.cu, NFFT2_2D_GPU: one child grid of 13 x 13 threads per
    point) is timed beside the library's: config 1 (64 x 64, 4096 uniform
    points, PCG64 seed 0) and a 65,536-point random subset of the polar
    raster (512 x 512).  Coordinates in grid units, complex64 values."""
    cases = []
    rng = np.random.default_rng(0)
    x = (rng.uniform(-0.5, 0.5, 4096) * 64).astype(np.float32)
    y = (rng.uniform(-0.5, 0.5, 4096) * 64).astype(np.float32)
    d = (rng.uniform(-1, 1, 4096) + 1j * rng.uniform(-1, 1, 4096)).astype(np.complex64)
    cases.append(("uniform_64x64_4096", 64, 64, x, y, d))
    wl = polar_raster()
    idx = np.sort(np.random.default_rng(65536).choice(wl["x1"].size, 65536, replace=False))
    cases.append(("polar_raster_512x512_subset_65536", 512, 512, (wl["x1"][idx] * 512).astype(np.float32),
                  (wl["x2"][idx] * 512).astype(np.float32), wl["f"][idx]))
    return cases


def reference_gpu_spread(reps: int = 5):
    """Time the reference's own GPU spreading (oracle/_ref: NFFT2_2D.cu
    compiled unchanged, host side restated) on small_spread_cases():
    the interpolation kernel with its child grids (CUDA events) and the whole
    NFFT2_2D_GPU call (host clock: per-call constants, allocations and
    synchronisations included).  Medians of `reps` calls after one warm-up."""
    try:
        import torch

        from oracle import ref_gpu
        if not torch.cuda.is_available():
            return {"unavailable": "no CUDA device"}
        if not ref_gpu.available():
            return {"unavailable": "oracle/_ref/nfft2_2d_ref.cubin was not built"}
        out = {}
        for name, N1, N2, x, y, d in small_spread_cases():
            dev = torch.device("cuda", 0)
            tx, ty, td = (torch.from_numpy(a).to(dev) for a in (x, y, d))
            ref_gpu.nfft2_2d_gpu(td, tx, ty, N1, N2)
            ti, tt = [], []
            for _ in range(reps):
                _, a, b = ref_gpu.nfft2_2d_gpu(td, tx, ty, N1, N2, timing=True)
                ti.append(a)
                tt.append(b)
            out[name] = {"interpolation_kernel_ms": statistics.median(ti), "call_ms": statistics.median(tt),
                         "points": int(x.size)}
        out["note"] = ("reference NFFT2_2D_GPU float overload (sigma 2, K 6) on the GPU: interpolation = "
                       "Interpolation_NFFT2_2D_GPUKernel with its per-point series_terms child grids (CUDA events); "
                       "call = the whole call by host clock")
        return out
    except Exception as e:  # the CPU line must still print
        return {"unavailable": f"{type(e).__name__}: {e}"}


def spread_small_cases(stream, reps: int = 5):
    """The library's type-1 spreading with the reference's sign on
    small_spread_cases(): the spread kernel (plan events, grid zeroing
    included) and the whole type-1 call (CUDA events on the plan's stream)."""
    import torch

    from miscellaneous_gb300.nfft import Plan
    dev = torch.device("cuda", torch.cuda.current_device())
    out = {}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for name, N1, N2, x, y, d in small_spread_cases():
        tx, ty, td = (torch.from_numpy(a).to(dev) for a in (x, y, d))
        F = torch.empty(N1 * N2, dtype=torch.complex64, device=dev)
        with Plan(N1, N2, sigma=2.0, K=6, precision="f32", stream=stream) as p:
            p.set_points(tx, ty, units="grid")
            p.spread_ref(td, out=F)
            p.enable_timing(True)
            ks, cs = [], []
            for _ in range(reps):
                ev0.record(stream)
                p.spread_ref(td, out=F)
                ev1.record(stream)
                ev1.synchronize()
                cs.append(ev0.elapsed_time(ev1))
                ks.append(p.timings()["spread_ms"])
            p.synchronize()
        out[name] = {"spread_kernel_ms": statistics.median(ks), "call_ms": statistics.median(cs),
                     "points": int(x.size)}
    out["note"] = ("nfft2d_spread_ref (type 1, sign -1, sigma 2, K 6) on the shapes the reference arm times the "
                   "reference's own GPU spreading on; spread = grid zeroing + spread kernel (plan events)")
    return out


def run_reference(args, wl):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build()
    M = wl["x1"].size
    # bounded sample per step: the full grid and as many points as keep a step under a second
    idx, _ = choose_cpu_sample(wl)
    m = idx.size
    for _ in range(args.warmup):
        cpu_reference_step(wl, idx)
    times = [cpu_reference_step(wl, idx) for _ in range(args.steps)]
    t = sum(times) / len(times)
    cb = {"unit": UNIT, "cores": oracle.get_threads(), "kind": "port"}
    if m < M:
        # t(m) = a + b m from a second, 4x smaller sample: the rate for all M points
        m2 = max(1, m // 4)
        idx2 = _cpu_sample(wl, np.random.default_rng(321), m2)
        t2 = statistics.median([cpu_reference_step(wl, idx2) for _ in range(3)])
        b = max((t - t2) / (m - m2), 0.0)
        a = max(t - b * m, 0.0)
        value = M / (a + b * M)
        cb.update(extrapolated=True, model={"grid_s": a, "per_point_s": b, "sample_points": m,
                                            "small_sample_points": m2, "small_sample_ms": t2 * 1e3})
        how = (f"{m} of {M} points with the full {wl['N1']}x{wl['N2']} grid per step (and {m2} points for the "
               f"model t(m) = a + b m); value = M / (a + b M)")
    else:
        value = m / t
        cb.update(extrapolated=False)
        how = f"all {M} points with the full {wl['N1']}x{wl['N2']} grid per step"
    cb.update(value=value, sample=(f"{how}; oracle/nfft2d_oracle.c restates NFFT1_2D.m (forward) and NFFT2_2D.m "
                                   "(spreading, sign +1), OpenMP over the host cores; the reference's MATLAB code "
                                   "cannot run on the host"))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": wl["config"], "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_reference_gpu:
        line["reference_gpu_spread"] = reference_gpu_spread()
    print(json.dumps(line))


def precision_study(args, wl, widths, x1, x2, F, f, stream, flush, torch):
    """The clustered configuration is a precision study across the window
    half-width: for each further w, a plan on the same resident points, the
    same timed forward + adjoint step (CUDA events, L2 flushed between
    steps) and the same subset accuracy."""
    from miscellaneous_gb300.nfft import Plan
    N1, N2, M = wl["N1"], wl["N2"], x1.numel()
    out = {}
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    f_out = torch.empty(M, dtype=torch.complex64, device=x1.device)
    F_out = torch.empty(N1 * N2, dtype=torch.complex64, device=x1.device)
    for K in widths:
        p = Plan(N1, N2, sigma=wl["sigma"], K=K, precision="f32", stream=stream)
        p.set_points(x1, x2, units="unit")
        for _ in range(args.warmup):
            p.forward(F, out=f_out)
            p.adjoint(f, out=F_out)
            flush.zero_()
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            ev0.record(stream)
            p.forward(F, out=f_out)
            p.adjoint(f, out=F_out)
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
            flush.zero_()
        p.synchronize()
        t = sum(ms) / len(ms)
        entry = {"ms_per_step": t, "value": M / (t * 1e-3), "unit": UNIT}
        if not args.no_accuracy:
            p.forward(F, out=f_out)
            p.synchronize()
            e_fwd, e_adj, nsub, _ = subset_accuracy(f_out, F, f, x1, x2, N1, N2, 65536, 7,
                                                    {"sigma": wl["sigma"], "K": K}, stream, torch)
            entry.update(rel_l2_forward=e_fwd, rel_l2_adjoint=e_adj, subset_points=nsub)
        out[f"w{K}"] = entry
        p.close()
    return out


def run_ours(args, wl):
    import torch
    import torch.distributed as dist

    from miscellaneous_gb300.nfft import Plan
    from miscellaneous_gb300.shard import ShardedPlan

    world, rank, local = dist_env()
    torch.cuda.set_device(local)  # before the process group: NCCL binds each rank to its device
    if world > 1:
        dist.init_process_group("nccl")
        # one transform of world * M points: each rank draws its own M points
        # (the workload's distribution, a rank-specific seed) and keeps them
        if wl["name"].startswith("clustered"):
            wl = clustered_config3(seed=3 + 1000 * rank, K=wl["K"], M=wl["x1"].size)
        elif wl["name"].startswith("polar"):
            wl = polar_raster(seed=2 + 1000 * rank, K=wl["K"])
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    N1, N2, M = wl["N1"], wl["N2"], wl["x1"].size
    G = int(round(wl["sigma"] * N1)) * int(round(wl["sigma"] * N2))

    x1 = torch.from_numpy(wl["x1"]).to(dev)
    x2 = torch.from_numpy(wl["x2"]).to(dev)
    F = torch.from_numpy(wl["F"]).to(dev).reshape(-1)
    f = torch.from_numpy(wl["f"]).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    sharded = ShardedPlan(N1, N2, sigma=wl["sigma"], K=wl["K"], precision="f32", stream=stream)
    plan = sharded.plan
    if args.fft_mode != "auto":
        plan.set_tuning(fft_mode={"cufft": 0, "pruned": 1, "fused": 2}[args.fft_mode])
    plan.set_points(x1, x2, units="unit")
    tuned = None
    if args.no_autotune and (args.gather_variant != "auto" or args.chunk):
        from miscellaneous_gb300 import _lib as _l
        gv = {"auto": -1, "tiled": _l.VARIANT_TILED, "direct": _l.VARIANT_DIRECT}[args.gather_variant]
        plan.set_tuning(gather_variant=gv, chunk=args.chunk or -1)
        plan.set_points(x1, x2, units="unit")
    if not args.no_autotune:
        from miscellaneous_gb300 import autotune
        tuned = autotune.tune(plan, x1, x2, F, f, use_cache=False)  # measured here, outside the timed region
    f_out = torch.empty(M, dtype=torch.complex64, device=dev)
    F_out = torch.empty(N1 * N2, dtype=torch.complex64, device=dev)
    if args.io_order == "binned":  # profiling runs of the binned order (the line's own arm stays in caller order)
        plan.set_tuning(io_order="binned")

    def step():
        sharded.forward(F, out=f_out)  # this rank's points, no collective
        sharded.adjoint(f, out=F_out)  # this rank's points, then the sum all-reduce (N > 1)

    # the timed steps run without the plan's per-stage events (recording them
    # costs ~10 % of a polar step); the stage breakdown comes from as many
    # further steps with them, after the timed region
    plan.enable_timing(False)
    for _ in range(args.warmup):
        step()
        flush.zero_()
    plan.synchronize()

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    stage = {k: 0.0 for k in ("pad", "fft_fwd", "halo_fill", "gather", "spread", "fold", "fft_adj", "crop")}
    step_ms = []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            ev0.record(stream)
            step()
            ev1.record(stream)
            ev1.synchronize()
            step_ms.append(ev0.elapsed_time(ev1))
            flush.zero_()  # L2 flush between timed steps, outside the events
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    plan.synchronize()
    plan.enable_timing(True)
    for _ in range(args.steps):
        step()
        plan.synchronize()
        t = plan.timings()  # the plan's own events on the launching stream
        stage["pad"] += t["pad_ms"]
        stage["fft_fwd"] += t["fft_type2_ms"]
        stage["halo_fill"] += t["halo_fill_ms"]
        stage["gather"] += t["gather_ms"]
        stage["spread"] += t["spread_ms"]
        stage["fold"] += t["fold_ms"]
        stage["fft_adj"] += t["fft_type1_ms"]
        stage["crop"] += t["crop_ms"]
        flush.zero_()
    plan.enable_timing(False)
    plan.set_tuning(io_order="caller")  # the checks and e2e below use the caller's order
    t_step = sum(step_ms) / len(step_ms)
    if world > 1:
        tt = torch.tensor([t_step], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())
    for k in stage:
        stage[k] /= args.steps
    value = world * M / (t_step * 1e-3)

    # ---- dominant kernel roofline ----
    peak, peak_kind = measured_peaks()
    alg_bytes = 20 * M + 8 * G  # algorithmic bytes: gather and spread both move 20 B/point + 8 B/cell
    dom = "gather" if stage["gather"] >= stage["spread"] else "spread"
    dom_ms = stage[dom]
    achieved = alg_bytes / (dom_ms * 1e-3) / 1e9
    ginfo = plan.info()
    kname = {"gather": "k_gather_tiled" if ginfo["gather_variant"] == 1 else "k_gather_direct",
             "spread": "k_spread_tiled" if ginfo["spread_variant"] == 1 else "k_spread_direct"}[dom]
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": dom_ms,
                "traffic": ncu_traffic(kname, wl["name"])}
    # the same kernel with the per-point arrays in the plan's binned order
    # (io_order binned): no random 8-byte accesses to f
    tb = ncu_traffic(kname + "_binned", wl["name"])
    if tb is not None:
        roofline["traffic_binned_io"] = tb
        roofline["traffic_note"] = ("traffic: caller-order f (random 8-byte accesses, one sector each); "
                                    "traffic_binned_io: f in the binned order (the binned_io arm)")

    # ---- e2e through the public API with pinned host buffers ----
    e2e = None
    if not args.no_e2e:
        hx1 = torch.from_numpy(wl["x1"]).pin_memory()
        hx2 = torch.from_numpy(wl["x2"]).pin_memory()
        hF = torch.from_numpy(wl["F"]).reshape(-1).pin_memory()
        hf = torch.from_numpy(wl["f"]).pin_memory()
        hf_out = torch.empty(M, dtype=torch.complex64).pin_memory()
        hF_out = torch.empty(N1 * N2, dtype=torch.complex64).pin_memory()
        dx1, dx2 = torch.empty_like(x1), torch.empty_like(x2)
        df = torch.empty_like(f)
        plan.enable_timing(False)
        # The link carries x1, x2, F and f up and f_out, F_out down.  The
        # binning needs the coordinates first, so they go first and alone
        # (concurrent uploads share the link); the library uploads the
        # page-locked F once they are read, while the rest of the binning
        # runs; f goes up on a second stream once those inputs are read,
        # while the forward runs, and f_out comes down on it while the
        # adjoint runs.  e2e_coords "direct": the binning pass reads the
        # page-locked coordinates over the link itself (set_points accepts
        # them), so the upload and the pass overlap; "copy": they are
        # copied first.
        cs = torch.cuda.Stream(device=dev)
        ev_sp, ev_in, ev_fwd, ev_out = (torch.cuda.Event() for _ in range(4))
        mode = {"direct": args.e2e_coords == "direct"}

        def e2e_step():
            if mode["direct"]:
                cx1, cx2 = hx1, hx2
            else:
                dx1.copy_(hx1, non_blocking=True)
                dx2.copy_(hx2, non_blocking=True)
                cx1, cx2 = dx1, dx2
            # binning + forward in one call: F goes up once the coordinates
            # are read, and the forward's pad and FFT run while the points
            # are binned; ev_sp marks the inputs read, after which f goes up
            # on the second stream
            plan.bin_and_forward(cx1, cx2, hF, units="unit", out=f_out, inputs_read=ev_sp)
            cs.wait_event(ev_sp)
            with torch.cuda.stream(cs):
                df.copy_(hf, non_blocking=True)
                ev_in.record(cs)
            ev_fwd.record(stream)
            stream.wait_event(ev_in)
            sharded.adjoint(df, out=F_out)
            cs.wait_event(ev_fwd)
            with torch.cuda.stream(cs):
                hf_out.copy_(f_out, non_blocking=True)
                ev_out.record(cs)
            hF_out.copy_(F_out, non_blocking=True)
            stream.wait_event(ev_out)

        # "auto": which coordinate path this machine's host link favours, from a
        # short untimed trial of each (the kernel-read path measured 3.88 ms
        # per config-3 step on some boxes and 4.8 ms on others, the copy
        # path 4.14 ms on all), like the kernel autotuner's trial
        trial = None
        if args.e2e_coords == "auto":
            trial = {}
            for m in ("direct", "copy"):
                mode["direct"] = m == "direct"
                for _ in range(2):
                    e2e_step()
                    plan.synchronize()
                ts = []
                for _ in range(3):
                    flush.zero_()
                    ev0.record(stream)
                    e2e_step()
                    ev1.record(stream)
                    ev1.synchronize()
                    ts.append(ev0.elapsed_time(ev1))
                    plan.synchronize()
                trial[m] = statistics.median(ts)
            mode["direct"] = trial["direct"] <= trial["copy"]
        for _ in range(args.warmup):
            e2e_step()
            plan.synchronize()
        torch.cuda.synchronize()
        e_ms = []
        for _ in range(args.steps):
            ev0.record(stream)
            e2e_step()
            ev1.record(stream)
            ev1.synchronize()
            e_ms.append(ev0.elapsed_time(ev1))
            plan.synchronize()  # the step's status (errors of the binning), outside the events
            flush.zero_()       # L2 flush between timed steps, outside the events
        te = sum(e_ms) / len(e_ms)
        if world > 1:
            tt = torch.tensor([te], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            te = float(tt.item())
        h2d = (hx1.numel() * 4 + hx2.numel() * 4 + hF.numel() * 8 + hf.numel() * 8)
        d2h = hf_out.numel() * 8 + hF_out.numel() * 8
        # the coordinates' upload alone (the part of the copies on the
        # critical path), for the breakdown
        cu_ms = []
        for _ in range(3):
            ev0.record(stream)
            dx1.copy_(hx1, non_blocking=True)
            dx2.copy_(hx2, non_blocking=True)
            ev1.record(stream)
            ev1.synchronize()
            cu_ms.append(ev0.elapsed_time(ev1))
        cu = statistics.median(cu_ms)
        e2e = {"value": world * M / (te * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": te,
               "ms_per_step_min_median_max": [min(e_ms), statistics.median(e_ms), max(e_ms)],
               "coords_upload_ms": cu, "coords_upload_gbs": (hx1.numel() + hx2.numel()) * 4 / (cu * 1e-3) / 1e9,
               "coords": "direct" if mode["direct"] else "copy", "coords_trial_ms": trial,
               "includes": "H2D of the coordinates (read by the binning pass over the link with coords "
                           "'direct', copied first with 'copy'; the faster of the two in an untimed trial), F and f; "
                           "binning + forward in one call (nfft2d_bin_and_forward with the page-locked F: F goes up "
                           "once the coordinates are read, the forward's pad and FFT run while the points are "
                           "binned), adjoint, D2H of f_out and F_out; f goes up once those inputs are read, f_out "
                           "comes down during the adjoint (second stream); the plan status is read and L2 is "
                           "flushed (256 MB written) after each step, outside the events"}
        # restore the resident plan state for the accuracy check
        plan.set_points(x1, x2, units="unit")

    # ---- accuracy vs FP64 NDFT (after timing, not timed) ----
    accuracy = None
    if not args.no_accuracy and rank == 0:
        plan.forward(F, out=f_out)
        plan.synchronize()
        e_fwd, e_adj, nsub, _ = subset_accuracy(f_out, F, f, x1, x2, N1, N2, 65536, 7,
                                                {"sigma": wl["sigma"], "K": wl["K"]}, stream, torch)
        accuracy = {"rel_l2_forward": e_fwd, "rel_l2_adjoint": e_adj, "subset_points": nsub,
                    "oracle": "FP64 NDFT (exact phase reduction) via torch complex128 on the GPU"}

    # ---- set_points on its own, and "set_points + execute" (after timing) ----
    plan.enable_timing(True)
    sp_ms = []
    for r in range(args.warmup + args.steps):
        flush.zero_()
        plan.set_points(x1, x2, units="unit")
        if r >= args.warmup:
            sp_ms.append(plan.timings()["sort_ms"])
    set_points_ms = sum(sp_ms) / len(sp_ms)

    # ---- cuFFT, timed on its own on the same grid (a second plan in cuFFT mode) ----
    cufft = None
    if plan.info()["fft_mode"] == 2:
        cplan = Plan(N1, N2, sigma=wl["sigma"], K=wl["K"], precision="f32", stream=stream)
        cplan.set_tuning(fft_mode=0)
        cplan.set_points(x1, x2, units="unit")
        cplan.enable_timing(True)
        ts = []
        for r in range(args.warmup + args.steps):
            cplan.forward(F, out=f_out)
            cplan.adjoint(f, out=F_out)
            if r >= args.warmup:
                ts.append(cplan.timings())
            flush.zero_()
        cplan.synchronize()
        cplan.close()
        avg = {k: sum(t[k] for t in ts) / len(ts) for k in ("pad_ms", "fft_type2_ms", "halo_fill_ms", "fold_ms",
                                                            "fft_type1_ms", "crop_ms")}
        cufft = {"fft_fwd_ms": avg["fft_type2_ms"], "fft_adj_ms": avg["fft_type1_ms"],
                 "fft_ms": avg["fft_type2_ms"] + avg["fft_type1_ms"],
                 "with_pad_fill_fold_crop_ms": sum(avg.values()),
                 "note": "cuFFT 2D plan on the same grid with the separate pad / halo fill / halo fold / crop "
                         "kernels; the line's own FFT is the fused passes"}

    study = None
    if wl["name"].startswith("clustered") and not args.no_precision_study and world == 1:
        study = precision_study(args, wl, [k for k in (4, 6, 8) if k != wl["K"]], x1, x2, F, f, stream, flush,
                                torch)
        study[f"w{wl['K']}"] = {"ms_per_step": t_step, "value": M / (t_step * 1e-3), "unit": UNIT}
        if accuracy is not None:
            study[f"w{wl['K']}"].update(rel_l2_forward=accuracy["rel_l2_forward"],
                                        rel_l2_adjoint=accuracy["rel_l2_adjoint"],
                                        subset_points=accuracy["subset_points"])
        study = dict(sorted(study.items()))

    # the same step with the per-point arrays in the plan's binned order (an
    # iterative solver keeps its vectors in that order): the gather writes and
    # the spread reads them contiguously instead of at random caller indices
    binned = None
    if world == 1:
        perm = plan.permutation().long()
        f_b = f[perm].contiguous()
        plan.set_tuning(io_order="binned")
        for _ in range(args.warmup):
            plan.forward(F, out=f_out)
            plan.adjoint(f_b, out=F_out)
            flush.zero_()
        torch.cuda.synchronize()
        bms = []
        for _ in range(args.steps):
            ev0.record(stream)
            plan.forward(F, out=f_out)
            plan.adjoint(f_b, out=F_out)
            ev1.record(stream)
            ev1.synchronize()
            bms.append(ev0.elapsed_time(ev1))
            flush.zero_()
        plan.set_tuning(io_order="caller")
        tb = sum(bms) / len(bms)
        binned = {"ms_per_step": tb, "value": M / (tb * 1e-3), "unit": UNIT,
                  "traffic": {k: ncu_traffic(k + "_binned", wl["name"]) for k in ("k_gather_direct", "k_spread_tiled")},
                  "note": "io_order binned (nfft2d_tuning): f in the plan's binned order, same points and grid; "
                          "traffic = DRAM bytes per launch from the committed ncu summary"}
        del f_b, perm

    small = spread_small_cases(stream) if rank == 0 and not args.no_reference_gpu else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_isolated(args)

    fused = plan.info()["fft_mode"] == 2
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(wl["config"], l2="256 MB buffer written between timed steps (working set %s L2)"
                           % ("<" if 8 * G + 36 * M < L2_BYTES else ">"),
                           points_prebinned=True,
                           parallelism=("points sharded: one transform of %d x M points, each rank gathers and "
                                        "spreads its own M, NCCL sum all-reduce of the N1 x N2 adjoint" % world)
                           if world > 1 else "single GPU",
                           tuning=(tuned or {}).get("tuning"), plan=plan.info()),
            "autotune_trials_ms": [{**c, "ms": round(ms, 4)} for c, ms in (tuned or {}).get("trials", [])] or None,
            "stages_ms": stage,
            "stages_note": STAGES_NOTE[fused],
            "forward_ms": stage["pad"] + stage["fft_fwd"] + stage["halo_fill"] + stage["gather"],
            "adjoint_ms": stage["spread"] + stage["fold"] + stage["fft_adj"] + stage["crop"],
            "fft_ms": (stage["pad"] + stage["fft_fwd"] + stage["fold"] + stage["fft_adj"]) if fused
            else stage["fft_fwd"] + stage["fft_adj"],
            "cufft_separate": cufft,
            "set_points_ms": set_points_ms,
            "set_points_plus_execute": {"value": world * M / ((t_step + set_points_ms) * 1e-3), "unit": UNIT,
                                        "ms_per_step": t_step + set_points_ms,
                                        "note": "binning timed by the plan's events, plus one execute step"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "accuracy": accuracy,
            "precision_study": study,
            "binned_io": binned,
            "spread_small_cases": small,
            "gpu_launches": 6 * args.steps,
            "gpu_launches_note": ("our kernels in the timed region per step: column FFT+pad, row FFT+fill, gather, "
                                  "spread, fold+row FFT, column FFT+crop") if fused else
                                 ("our kernels in the timed region per step: pad, halo_fill, gather, spread, fold, "
                                  "crop (cuFFT kernels not counted)"),
            "clocks": clocks.summary(),
        }
        print(json.dumps(line))
    plan.close()
    if world > 1:
        dist.destroy_process_group()


def run_lsq(args, wl):
    """Config 5: one gradient evaluation of L = ||A(f; x) - y||^2 per step --
    r = A f - y (forward), dL/df = A^H (2 r) (adjoint), dL/dx = Re(conj(2 r) dA f/dx)
    (coordinate gradient) -- on resident data.  value = points / step time."""
    import torch

    from miscellaneous_gb300.nfft import Plan
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    N1, N2, M = wl["N1"], wl["N2"], wl["x1"].size
    x1 = torch.from_numpy(wl["x1"]).to(dev)
    x2 = torch.from_numpy(wl["x2"]).to(dev)
    plan = Plan(N1, N2, sigma=wl["sigma"], K=wl["K"], stream=stream)
    plan.set_points(x1, x2)
    y = plan.forward(torch.from_numpy(wl["f_true"]).to(dev).reshape(-1)) + torch.from_numpy(wl["noise"]).to(dev)
    F = torch.from_numpy(wl["F"]).to(dev).reshape(-1)
    r = torch.empty(M, dtype=torch.complex64, device=dev)
    gF = torch.empty(N1 * N2, dtype=torch.complex64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def step():
        plan.forward(F, out=r)
        r.sub_(y).mul_(2.0)
        plan.adjoint(r, out=gF)
        return plan.grad_x(F, r)

    for _ in range(args.warmup):
        step()
        flush.zero_()
    torch.cuda.synchronize()
    ms = []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            ev0.record(stream)
            step()
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
            flush.zero_()
    t = sum(ms) / len(ms)
    # sanity of the gradient direction: one steepest-descent step on f with
    # the exact line search t = Re<A g, r> / ||A g||^2 must lower the loss
    plan.forward(F, out=r)
    r.sub_(y)
    loss0 = float(torch.sum(torch.abs(r) ** 2))
    plan.adjoint(2.0 * r, out=gF)
    Ag = plan.forward(gF)
    t_ls = float(torch.real(torch.vdot(Ag, r))) / float(torch.sum(torch.abs(Ag) ** 2))
    plan.forward(F - t_ls * gF, out=r)
    loss1 = float(torch.sum(torch.abs(r - y) ** 2))
    plan.synchronize()
    # accuracy against FP64 sums on a 65,536-point subset: forward, adjoint,
    # and the coordinate gradient (v = 2 r; df/dx1 = sum_k F_k (-2 pi i k1) e_k(x))
    accuracy = None
    if not args.no_accuracy:
        f_fwd = plan.forward(F)
        v = 2.0 * (f_fwd - y)
        g1, g2 = plan.grad_x(F, v)
        plan.synchronize()
        e_fwd, e_adj, nsub, idx = subset_accuracy(f_fwd, F, v, x1, x2, N1, N2, 65536, 11,
                                                  {"sigma": wl["sigma"], "K": wl["K"]}, stream, torch)
        Fm = F.reshape(N1, N2).to(torch.complex128)
        k1 = (torch.arange(N1, device=dev, dtype=torch.float64) - N1 // 2)[:, None]
        k2 = (torch.arange(N2, device=dev, dtype=torch.float64) - N2 // 2)[None, :]
        d1 = ndft_type2_subset(Fm * (-2j * math.pi) * k1, x1, x2, idx, -1, torch)
        d2 = ndft_type2_subset(Fm * (-2j * math.pi) * k2, x1, x2, idx, -1, torch)
        vs = v[idx].to(torch.complex128)
        r1, r2 = torch.real(vs.conj() * d1), torch.real(vs.conj() * d2)
        e_grad = float(torch.linalg.vector_norm(torch.cat([g1[idx].double() - r1, g2[idx].double() - r2])) /
                       torch.linalg.vector_norm(torch.cat([r1, r2])))
        accuracy = {"rel_l2_forward": e_fwd, "rel_l2_adjoint": e_adj, "rel_l2_grad_x": e_grad,
                    "subset_points": nsub,
                    "oracle": "FP64 NDFT and its coordinate derivative via torch complex128 on the GPU"}
    line = {"metric": METRIC, "value": M / (t * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(wl["config"], l2="256 MB buffer written between timed steps",
                           step="forward + residual + adjoint (dL/df) + coordinate gradient (dL/dx)"),
            "loss_before": loss0, "loss_after_one_step": loss1, "accuracy": accuracy, "clocks": clocks.summary()}
    print(json.dumps(line))
    plan.close()


def knab_cpu_step(wl, rows):
    import oracle
    t0 = time.perf_counter()
    oracle.knab_nfft2d(0.0, wl["rho_in"], wl["cos_in"], wl["data"], wl["rho_out"][:rows], wl["cos_out"][:rows],
                       wl["B1"], wl["B2"])
    return time.perf_counter() - t0


def knab_cpu_baseline(wl, target_s: float = 15.0, steps: int | None = None):
    """The oracle's restatement of knabNFFT2D on the first `rows` output rows
    (the full raster FFT and NFFT grid; a block of whole rows keeps the
    detected oversampling of the full output raster).  t(m) = a + b m from
    two block sizes gives the rate for the full output raster."""
    import oracle
    oracle.build()
    L1, L2 = wl["rho_out"].shape
    rows = 8
    dt = knab_cpu_step(wl, rows)
    while rows < L1 and dt < 1.0:  # grow until the per-point work stands out of the fixed FFT cost
        rows = min(L1, rows * 4)
        dt = knab_cpu_step(wl, rows)
    n = steps if steps is not None else max(1, min(20, int(target_s / max(dt, 1e-3))))
    t = statistics.median([knab_cpu_step(wl, rows) for _ in range(n)])
    M = L1 * L2
    out = {"unit": UNIT, "cores": oracle.get_threads(), "kind": "port", "ms_per_step": t * 1e3,
           "points": rows * L2, "sample_rate": rows * L2 / t}
    if rows < L1:
        r2 = max(1, rows // 4)
        t2 = statistics.median([knab_cpu_step(wl, r2) for _ in range(max(3, n // 2))])
        b = max((t - t2) / ((rows - r2) * L2), 0.0)
        a = max(t - b * rows * L2, 0.0)
        out["value"] = M / (a + b * M)
        out["extrapolated"] = True
        out["model"] = {"fixed_s": a, "per_point_s": b, "small_sample_points": r2 * L2, "small_sample_ms": t2 * 1e3}
        how = f"the first {rows} and {r2} of {L1} output rows (x {L2})"
    else:
        out["value"] = M / t
        how = f"all {L1} x {L2} outputs"
    out["sample"] = (f"{how}, full {wl['data'].shape[0]}x{wl['data'].shape[1]} raster; median of {n} steps; "
                     "oracle/nfft2d_oracle.c restating knabNFFT2D.m, KnabWindow.m and NFFT1_2D.m (OpenMP)")
    return out


def run_knab_reference(args, wl):
    _, rank, _ = dist_env()
    if rank != 0:
        return
    cb = knab_cpu_baseline(wl, steps=max(1, args.steps))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": wl["config"],
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_knab(args, wl):
    """One step = one regridding of the raster onto the bound output raster:
    raster FFT, windowed pad, oversampled FFT, halo fill, gather (the
    extrapolation fill has nothing to do: every output is inside)."""
    import torch

    from miscellaneous_gb300 import knab
    from miscellaneous_gb300._lib import Timings, load
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    L1, L2 = wl["rho_out"].shape
    M = L1 * L2
    rho_out = torch.from_numpy(wl["rho_out"]).to(dev)
    cos_out = torch.from_numpy(wl["cos_out"]).to(dev)
    data = torch.from_numpy(wl["data"]).to(dev)
    r = knab.Regridder(wl["rho_in"], wl["cos_in"], wl["B1"], wl["B2"], precision="f32", stream=stream)
    r.set_points(rho_out, cos_out)
    out = torch.empty(L1, L2, dtype=torch.complex64, device=dev)
    lib = load()
    ph = r.plan_handle()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(args.warmup):
        r(data, 0.0, out=out)
        flush.zero_()
    torch.cuda.synchronize()
    ms, stage = [], {"pad": 0.0, "fft": 0.0, "halo_fill": 0.0, "gather": 0.0}
    tm = Timings()
    # timed without the plan's per-stage events; the stage breakdown comes
    # from as many further steps with them
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            ev0.record(stream)
            r(data, 0.0, out=out)
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
            flush.zero_()
    lib.nfft2d_enable_timing(ph, 1)
    for _ in range(args.steps):
        r(data, 0.0, out=out)
        r.synchronize()
        lib.nfft2d_get_timings(ph, ctypes.byref(tm))
        stage["pad"] += tm.pad_ms
        stage["fft"] += tm.fft_type2_ms
        stage["halo_fill"] += tm.halo_fill_ms
        stage["gather"] += tm.gather_ms
        flush.zero_()
    t = sum(ms) / len(ms)
    for k in stage:
        stage[k] /= args.steps
    stage["raster_fft_and_launch"] = max(t - sum(stage.values()), 0.0)
    lib.nfft2d_enable_timing(ph, 0)
    info = r.info()
    G = info["N1"] * info["N2"] * 4  # sigma^2 N1 N2 oversampled cells
    peak, peak_kind = measured_peaks()
    alg = 20 * M + 8 * G
    roofline = {"bound": "hbm", "kernel": "gather", "achieved": alg / (stage["gather"] * 1e-3) / 1e9, "peak": peak,
                "unit": "GB/s", "frac": alg / (stage["gather"] * 1e-3) / 1e9 / peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)", "algorithmic_bytes_per_launch": alg,
                "launch_ms": stage["gather"], "traffic": None}
    # accuracy: the exact trigonometric sum of the same windowed spectrum
    # (torch complex128 on the GPU) on 65,536 random outputs
    accuracy = None
    if not args.no_accuracy:
        Gn, kgn = knab.KnabWindow(info["T1"], wl["B1"], 18, info["Ncols"])
        Gm, kgm = knab.KnabWindow(info["T2"], wl["B2"], 18, info["Nrows"])
        N1, N2 = info["N1"], info["N2"]
        E = torch.fft.fft2(data.to(torch.complex128))
        S = torch.zeros(N1, N2, dtype=torch.complex128, device=dev)
        i1 = torch.arange(-kgm, kgm + 1, device=dev)
        i2 = torch.arange(-kgn, kgn + 1, device=dev)
        Ew = E[i1.remainder(info["Nrows"])][:, i2.remainder(info["Ncols"])]
        S[N1 // 2 - kgm:N1 // 2 + kgm + 1, N2 // 2 - kgn:N2 // 2 + kgn + 1] = (
            Ew * torch.from_numpy(Gm).to(dev)[:, None] * torch.from_numpy(Gn).to(dev)[None, :])
        g = torch.Generator(device="cpu").manual_seed(7)
        idx = torch.randperm(M, generator=g)[:65536].to(dev)
        x1 = ((cos_out.reshape(-1) - wl["cos_in"][0]) / (info["Nrows"] * info["T2"]))
        x2 = ((rho_out.reshape(-1) - wl["rho_in"][0]) / (info["Ncols"] * info["T1"]))
        ref = ndft_type2_subset(S, x1, x2, idx, +1, torch)
        accuracy = {"rel_l2": rel_l2(out.reshape(-1)[idx], ref, torch), "subset_points": 65536,
                    "oracle": "exact sum of the Knab-windowed spectrum, torch complex128 on the GPU"}
    e2e = None
    if not args.no_e2e:
        hd = torch.from_numpy(wl["data"]).pin_memory()
        hout = torch.empty(L1, L2, dtype=torch.complex64).pin_memory()
        hro = torch.from_numpy(wl["rho_out"]).pin_memory()
        hco = torch.from_numpy(wl["cos_out"]).pin_memory()
        dd = torch.empty_like(data)

        def e2e_step():
            rho_out.copy_(hro, non_blocking=True)
            cos_out.copy_(hco, non_blocking=True)
            dd.copy_(hd, non_blocking=True)
            r.set_points(rho_out, cos_out)
            r(dd, 0.0, out=out)
            hout.copy_(out, non_blocking=True)

        for _ in range(args.warmup):
            e2e_step()
        torch.cuda.synchronize()
        es = []
        for _ in range(args.steps):
            ev0.record(stream)
            e2e_step()
            ev1.record(stream)
            ev1.synchronize()
            es.append(ev0.elapsed_time(ev1))
            flush.zero_()  # L2 flush between timed steps, outside the events
        te = sum(es) / len(es)
        e2e = {"value": M / (te * 1e-3), "unit": UNIT, "ms_per_step": te,
               "h2d_bytes_per_step": hd.numel() * 8 + hro.numel() * 8 * 2, "d2h_bytes_per_step": hout.numel() * 8,
               "includes": "H2D raster + output coordinates, set_points (extent, masks, binning), regrid, D2H; "
                           "L2 flushed (256 MB written) after each step, outside the events"}
    cpu = None if args.no_cpu_baseline else knab_cpu_baseline(wl)
    line = {"metric": METRIC, "value": M / (t * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(wl["config"], l2="256 MB buffer written between timed steps", knab=info),
            "stages_ms": stage, "roofline": roofline, "accuracy": accuracy, "e2e": e2e, "cpu_baseline": cpu,
            "gpu_launches": 3 * args.steps,
            "gpu_launches_note": "our kernels per step: knab pad, halo fill, gather (+ cuFFT x2, not counted), "
                                 "extrapolation fill skipped (no masked lines)",
            "clocks": clocks.summary()}
    print(json.dumps(line))
    r.close()


def run_batch(args, wl):
    """Config 4: the batched graph launch vs one transform per launch (the
    library's own single-transform path with pre-created plans)."""
    import torch

    from miscellaneous_gb300.nfft import Batch, Plan
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    g = torch.Generator(device=dev).manual_seed(wl["seed"])
    sizes = [(it["N"], it["N"]) for it in wl["items"]]
    x1s = [torch.rand(it["M"], device=dev, generator=g) - 0.5 for it in wl["items"]]
    x2s = [torch.rand(it["M"], device=dev, generator=g) - 0.5 for it in wl["items"]]
    Fs = [torch.randn(n1 * n2, dtype=torch.complex64, device=dev, generator=g) for n1, n2 in sizes]
    fs = [torch.randn(it["M"], dtype=torch.complex64, device=dev, generator=g) for it in wl["items"]]
    f_out = [torch.empty(it["M"], dtype=torch.complex64, device=dev) for it in wl["items"]]
    F_out = [torch.empty(n1 * n2, dtype=torch.complex64, device=dev) for n1, n2 in sizes]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    total = sum(it["M"] for it in wl["items"])
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(step):
        for _ in range(args.warmup):
            step()
            flush.zero_()
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            ev0.record(stream)
            step()
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
            flush.zero_()
        return sum(ms) / len(ms)

    batch = Batch(sizes, sigma=wl["sigma"], K=wl["K"], stream=stream)
    batch.set_points(x1s, x2s)

    def batched():
        batch.forward(Fs, f_out)
        batch.adjoint(fs, F_out)

    t_batch = timed(batched)
    plans = []
    for (n1, n2), a, b in zip(sizes, x1s, x2s):
        p = Plan(n1, n2, sigma=wl["sigma"], K=wl["K"], stream=stream)
        p.set_points(a, b)
        plans.append(p)

    def sequential():
        for p, F, fo in zip(plans, Fs, f_out):
            p.forward(F, out=fo)
        for p, f, Fo in zip(plans, fs, F_out):
            p.adjoint(f, out=Fo)

    t_seq = timed(sequential)
    batch.synchronize()
    # what the sequential arm is made of: each transform's kernel time (its
    # plan's stage events) against the arm's wall time; the difference is
    # the launch gaps that batching can remove
    for p in plans:
        p.enable_timing(True)
    per = []
    for _ in range(3):
        for i, (p, F, fo) in enumerate(zip(plans, Fs, f_out)):
            p.forward(F, out=fo)
            p.synchronize()
            tf = p.timings()
            p.adjoint(fs[i], out=F_out[i])
            p.synchronize()
            ta = p.timings()
            k = (tf["pad_ms"] + tf["fft_type2_ms"] + tf["halo_fill_ms"] + tf["gather_ms"] + ta["spread_ms"]
                 + ta["fold_ms"] + ta["fft_type1_ms"] + ta["crop_ms"])
            if len(per) <= i:
                per.append([])
            per[i].append(k)
    for p in plans:
        p.enable_timing(False)
    kern = [statistics.median(v) for v in per]
    table = {}
    for (n1, _), it, k in zip(sizes, wl["items"], kern):
        row = table.setdefault(str(n1), {"transforms": 0, "points": 0, "kernel_ms": 0.0})
        row["transforms"] += 1
        row["points"] += it["M"]
        row["kernel_ms"] += k
    breakdown = {"kernel_ms_sum": sum(kern), "sequential_wall_ms": t_seq,
                 "launch_gap_share": max(0.0, 1.0 - sum(kern) / t_seq),
                 "batched_over_kernel_sum": t_batch / sum(kern), "by_grid_size": table,
                 "note": "kernel_ms = the transform's stage events (pad, FFTs, fill, gather, spread, fold, crop) "
                         "timed one transform at a time; batching can remove at most the launch gaps"}
    accuracy = None
    if not args.no_accuracy:
        # the batched results themselves: forward on point subsets of a few
        # transforms, adjoint of the transforms with the fewest points
        # against the full FP64 type-1 sum
        batched()
        batch.synchronize()
        order = sorted(range(len(sizes)), key=lambda t: wl["items"][t]["M"])
        fwd_ts = sorted(set([order[0], order[len(order) // 2], order[-1], len(order) // 3]))
        e_fwd = 0.0
        for t in fwd_ts:
            n1, n2 = sizes[t]
            gsub = torch.Generator(device="cpu").manual_seed(100 + t)
            idx = torch.randperm(x1s[t].numel(), generator=gsub)[:16384].to(dev)
            ref = ndft_type2_subset(Fs[t].reshape(n1, n2), x1s[t], x2s[t], idx, -1, torch)
            e_fwd = max(e_fwd, rel_l2(f_out[t][idx], ref, torch))
        adj_ts = [t for t in order if wl["items"][t]["M"] * sizes[t][0] * sizes[t][1] <= 4e10][:3]
        e_adj = 0.0
        for t in adj_ts:
            n1, n2 = sizes[t]
            ref = ndft_type1(fs[t], x1s[t], x2s[t], n1, n2, +1, torch)
            e_adj = max(e_adj, rel_l2(F_out[t], ref, torch))
        accuracy = {"rel_l2_forward_max": e_fwd, "forward_transforms": fwd_ts, "forward_subset_points": "min(M, 16384)",
                    "rel_l2_adjoint_max": e_adj, "adjoint_transforms": adj_ts,
                    "oracle": "FP64 NDFT via torch complex128 on the GPU (adjoint: all points of the transform)"}
    line = {"metric": METRIC, "value": total / (t_batch * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_batch, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(wl["config"], l2="256 MB buffer written between timed steps"),
            "sequential_ms_per_step": t_seq, "batched_speedup": t_seq / t_batch,
            "sequential_breakdown": breakdown,
            "sequential": "one forward + one adjoint per transform through pre-created single-transform plans",
            "batched": "nfft2d_batch_forward + nfft2d_batch_adjoint, stage sequence replayed as a CUDA graph",
            "accuracy": accuracy}
    print(json.dumps(line))
    for p in plans:
        p.close()
    batch.close()


FFBP_METRIC = "FFBP SAR image: NU points/s (leaf NFFT1_1D points + Knab-regridded points) per image"


def ffbp_cpu_rate():
    """The oracle's restated FFBP (oracle/ffbp.py, FP64, OpenMP C kernels) on
    an 8-pulse, 64-sample, 32 x 32 point-target scene: points per second
    counted as the library counts them."""
    import oracle
    from oracle import ffbp as F
    oracle.build()
    data, sar = F.point_target_scene(Np=8, nf=64, Nx=32, R=2e3, step=0.08)
    import torch
    pts = None
    if torch.cuda.is_available():  # the work count of the same scene, from the library
        from miscellaneous_gb300.sar import FFBP
        st = {}
        FFBP(data, 1, 8, c=sar["c"], fc=sar["fc"], BW=sar["BW"], f2=sar["f2"], precision="f64", stats=st)
        pts = st["leaf_points"] + st["regrid_points"]
    F.ffbp(data, sar, 1, 8)
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        F.ffbp(data, sar, 1, 8)
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    return {"seconds_per_image": t, "points": pts, "value": (pts / t) if pts else None, "unit": UNIT,
            "cores": oracle.get_threads(), "kind": "port", "extrapolated": False,
            "sample": "8 pulses, 64 frequency samples, 32 x 32 scene at 2 km (the largest 8-pulse scene the "
                      "reference's recursion can run), median of 3 images; oracle/ffbp.py over the C restatements "
                      "of knabNFFT2D.m and NFFT1_1D.m"}


def run_ffbp(args, wl):
    import torch

    from miscellaneous_gb300.sar import FFBP, polar_grid
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    data, sar, Np = wl["data"], wl["sar"], wl["Np"]
    rho, cosa = polar_grid(data, 1)
    kw = dict(c=sar["c"], fc=sar["fc"], BW=sar["BW"], f2=sar["f2"], stream=stream)
    dev_data = dict(data, phdata=torch.from_numpy(data["phdata"]).to(dev))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    st = {}
    for _ in range(args.warmup):
        FFBP(dev_data, 1, Np, precision="f32", stats=st, **kw)
    torch.cuda.synchronize()
    ms = []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            ev0.record(stream)
            im = FFBP(dev_data, 1, Np, precision="f32", **kw)
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
    t = statistics.median(ms)
    pts = st["leaf_points"] + st["regrid_points"]
    im64 = FFBP(dev_data, 1, Np, precision="f64", **kw)
    a, b = im.to(torch.complex128), im64
    m = ~torch.isnan(b.real)
    err = float(torch.linalg.vector_norm((a - b)[m]) / torch.linalg.vector_norm(b[m]))
    cpu = None if args.no_cpu_baseline else ffbp_cpu_rate()
    line = {"metric": FFBP_METRIC, "value": pts / (t * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": wl["config"], "work": st,
            "images_per_s": 1e3 / t,
            "accuracy": {"rel_l2_f32_vs_f64": err, "nan_pixels": int((~m).sum()),
                         "note": "FP32 data (FP64 coordinates and phases) against the library's FP64 image; the FP64 "
                                 "path matches the oracle's restated recursion to 2e-12 (tests/test_gpu_ffbp.py)"},
            "cpu_baseline": cpu, "clocks": clocks.summary(),
            "step": "one whole image: host recursion, plan and regridder set-up, every kernel (CUDA events around "
                    "the synchronous call)"}
    print(json.dumps(line))


def run_ffbp_reference(args, wl):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    cb = ffbp_cpu_rate()
    value = cb["value"] if cb["value"] is not None else 1.0 / cb["seconds_per_image"]
    line = {"impl": "reference", "metric": FFBP_METRIC, "value": value,
            "unit": UNIT if cb["value"] is not None else "images/s", "n_gpus": world, "steps": 3,
            "warmup": 1, "ms_per_step": cb["seconds_per_image"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": wl["config"], "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


TYPE3_METRIC = "type-3 2D NUFFT: NU points/s (input points + output frequencies) per transform"


def type3_cpu_rate(wl, m: int = 1 << 16, reps: int = 3):
    """The oracle's restatement of NUFFT_2D_CPU (OpenMP on all host cores) on
    m points and m frequencies drawn from the workload and on m/4 of each,
    t(m) = a + b m; value = the model's rate for the full sizes.  The
    reference's own NFFT3_2D_C.cpp needs Intel MKL and FFTW (absent)."""
    import oracle
    oracle.build()
    M, N = wl["x"].size, wl["s"].size
    rng = np.random.default_rng(1234)

    def step(k):
        i = np.sort(rng.choice(M, k, replace=False))
        j = np.sort(rng.choice(N, k, replace=False))
        args = (wl["x"][i], wl["y"][i], wl["f"][i].astype(np.complex128), wl["s"][j], wl["t"][j])
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            _, info = oracle.nufft3_2d(*args, eps=wl["eps"])
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts), info

    t1, info = step(m)
    t2, _ = step(m // 4)
    b = max((t1 - t2) / (2 * (m - m // 4)), 0.0)
    a = max(t1 - b * 2 * m, 0.0)
    value = (M + N) / (a + b * (M + N))
    return {"value": value, "unit": UNIT, "cores": oracle.get_threads(), "kind": "port", "extrapolated": True,
            "model": {"fixed_s": a, "per_point_s": b, "sample": m, "small_sample": m // 4,
                      "sample_ms": t1 * 1e3, "grid": [info["Mry"], info["Mrx"]], "msp": info["msp"]},
            "sample": (f"{m} points + {m} frequencies drawn from the workload (and {m // 4} + {m // 4}), median of "
                       f"{reps}; oracle/nfft2d_oracle.c restates NUFFT_2D_CPU (NFFT3_2D_C.cpp:199-312), FP64, "
                       "OpenMP; the reference's own code needs Intel MKL and FFTW, absent here")}


def run_type3(args, wl):
    import torch

    from miscellaneous_gb300.nufft3 import NUFFT_2D
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    M, N = wl["x"].size, wl["s"].size
    x, y, s, t = (torch.from_numpy(wl[k]).to(dev) for k in ("x", "y", "s", "t"))
    f = torch.from_numpy(wl["f"]).to(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        NUFFT_2D(x, y, s, t, f, wl["eps"], stream=stream)
    torch.cuda.synchronize()
    ms = []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            ev0.record(stream)
            F = NUFFT_2D(x, y, s, t, f, wl["eps"], stream=stream)
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
    tm = statistics.median(ms)
    # e2e: host arrays in, F out
    e2e = None
    if not args.no_e2e:
        hx, hy, hs, ht = (torch.from_numpy(wl[k]).pin_memory() for k in ("x", "y", "s", "t"))
        hf = torch.from_numpy(wl["f"]).pin_memory()
        hF = torch.empty(N, dtype=torch.complex64).pin_memory()
        dx, dy, ds, dt_ = (torch.empty_like(v) for v in (x, y, s, t))
        df = torch.empty_like(f)
        em = []
        for r in range(args.warmup + args.steps):
            flush.zero_()
            ev0.record(stream)
            for d, h in ((dx, hx), (dy, hy), (df, hf), (ds, hs), (dt_, ht)):
                d.copy_(h, non_blocking=True)
            Fd = NUFFT_2D(dx, dy, ds, dt_, df, wl["eps"], stream=stream)
            hF.copy_(Fd, non_blocking=True)
            ev1.record(stream)
            ev1.synchronize()
            if r >= args.warmup:
                em.append(ev0.elapsed_time(ev1))
        te = statistics.median(em)
        e2e = {"value": (M + N) / (te * 1e-3), "unit": UNIT, "ms_per_step": te,
               "h2d_bytes_per_step": 16 * M + 8 * M + 16 * N, "d2h_bytes_per_step": 8 * N}
    accuracy = None
    if not args.no_accuracy:
        # exact FP64 sums for 512 of the frequencies (torch complex128 on the GPU)
        sel = torch.from_numpy(np.random.default_rng(99).choice(N, 512, replace=False)).to(dev)
        fe = f.to(torch.complex128)
        ref = torch.empty(512, dtype=torch.complex128, device=dev)
        for c0 in range(0, 512, 32):
            k = sel[c0:c0 + 32]
            ph = torch.outer(s[k], x) + torch.outer(t[k], y)
            ref[c0:c0 + 32] = torch.polar(torch.ones_like(ph), -ph) @ fe
        got = F[sel].to(torch.complex128)
        accuracy = {"rel_l2": float(torch.linalg.vector_norm(got - ref) / torch.linalg.vector_norm(ref)),
                    "frequencies_checked": 512, "oracle": "exact FP64 sum over all points (torch complex128)"}
    cpu = None if args.no_cpu_baseline else type3_cpu_rate(wl)
    line = {"metric": TYPE3_METRIC, "value": (M + N) / (tm * 1e-3), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tm, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(wl["config"], l2="256 MB buffer written before each timed call"),
            "step": "one nfft2d_nufft3_2d call (extents, grid allocation, spread, cuFFT, gather; synchronous), "
                    "CUDA events around it",
            "accuracy": accuracy, "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks.summary()}
    print(json.dumps(line))


def run_type3_reference(args, wl):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    cb = type3_cpu_rate(wl)
    line = {"impl": "reference", "metric": TYPE3_METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": world,
            "steps": 3, "warmup": 0, "ms_per_step": (wl["x"].size + wl["s"].size) / cb["value"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": wl["config"], "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="clustered")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="reference arm: skip timing the reference's own GPU spreading (oracle/_ref)")
    ap.add_argument("--no-precision-study", action="store_true",
                    help="clustered workload: skip the other window half-widths (w 4, 6, 8)")
    ap.add_argument("--fft-mode", choices=["auto", "cufft", "pruned", "fused"], default="auto",
                    help="oversampled FFT: auto (fused passes below 2048^2 cells, else cuFFT), cuFFT 2D plan, "
                         "cuFFT passes, fused")
    ap.add_argument("--io-order", choices=["caller", "binned"], default="caller",
                    help="per-point arrays of the timed steps in the caller's or the plan's binned order")
    ap.add_argument("--e2e-coords", choices=["auto", "direct", "copy"], default="auto",
                    help="e2e: the binning reads the page-locked coordinates over the link (direct) or after "
                         "a copy (copy); auto picks the faster by an untimed trial of each")
    ap.add_argument("--gather-variant", choices=["auto", "tiled", "direct"], default="auto",
                    help="with --no-autotune: the gather kernel to use (default: the plan's default)")
    ap.add_argument("--chunk", type=int, default=None,
                    help="with --no-autotune: points per work item (default: the plan's default, 256)")
    ap.add_argument("--points", type=int, default=None,
                    help="clustered workload only: this many points instead of 2^24 (same grid and seed), "
                         "for profiler captures of the same kernels on a smaller working set")
    ap.add_argument("--K", type=int, default=None,
                    help="window half-width for the clustered and polar workloads (2..8; default 6)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.points is not None and args.workload != "clustered":
        ap.error("--points applies to the clustered workload only")
    if args.workload == "clustered":
        kw = {} if args.K is None else {"K": args.K}
        if args.points is not None:
            kw["M"] = args.points
        wl = clustered_config3(**kw)
    else:
        wl = (WORKLOADS[args.workload](K=args.K) if (args.workload == "polar" and args.K)
              else WORKLOADS[args.workload]())
    if args.workload == "ffbp":
        if args.impl == "reference":
            run_ffbp_reference(args, wl)
        else:
            run_ffbp(args, wl)
        return
    if args.workload == "type3":
        if args.impl == "reference":
            run_type3_reference(args, wl)
        else:
            run_type3(args, wl)
        return
    if args.workload == "knab":
        if args.impl == "reference":
            run_knab_reference(args, wl)
        else:
            run_knab(args, wl)
    elif args.workload == "lsq":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the least-squares workload has no reference counterpart"}))
            return
        run_lsq(args, wl)
    elif args.workload == "pso":
        if args.impl == "reference":
            run_pso_reference(args, wl)
        else:
            run_pso(args, wl)
    elif args.workload == "batch":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batch workload has no reference counterpart"}))
            return
        run_batch(args, wl)
    elif args.impl == "reference":
        run_reference(args, wl)
    else:
        run_ours(args, wl)


if __name__ == "__main__":
    main()
