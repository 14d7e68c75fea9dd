"""Autotuner for the bin / work-item parameters of a plan.

The best settings depend on the point distribution (uniform, polar,
clustered) and the grid size, so they are measured, not guessed: for each
candidate the tuner times forward + adjoint on the caller's own points with
the plan's CUDA events and keeps the fastest.  Results are cached in a JSON
file keyed by (N1, N2, sigma, K, log2 M, GPU name), so later plans of the
same shape reuse them without measuring.

Candidates: the gather variant (TMA-tiled shared-memory patches, or direct
L1/L2 reads of the padded grid) and the work-item size (points per tile work
item; above 512 points the spread keeps items of 512, the tiled gather takes
the larger ones).  The tile edge stays at 16, which the register-resident
spread needs.
"""
from __future__ import annotations

import json
import math
import os
import threading

from . import _lib

_DEFAULT_CANDIDATES = (
    dict(gather_variant=_lib.VARIANT_TILED, chunk=256),
    dict(gather_variant=_lib.VARIANT_TILED, chunk=128),
    dict(gather_variant=_lib.VARIANT_TILED, chunk=512),
    dict(gather_variant=_lib.VARIANT_TILED, chunk=2048),  # the spread then cuts its own 512-point items
    dict(gather_variant=_lib.VARIANT_DIRECT, chunk=256),
    dict(gather_variant=_lib.VARIANT_DIRECT, chunk=128),
)

_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("NFFT2D_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "nfft2d_gb300", "autotune.json"))


def cache_key(N1: int, N2: int, sigma: float, K: int, M: int, device_name: str) -> str:
    mb = int(math.floor(math.log2(M))) if M > 0 else 0
    return f"{N1}x{N2}|s{sigma:g}|K{K}|M2^{mb}|{device_name}"


def load_cache(path: str | None = None) -> dict:
    path = path or cache_path()
    try:
        with open(path) as fh:
            data = json.load(fh)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def store(key: str, tuning: dict, ms: float, path: str | None = None) -> None:
    path = path or cache_path()
    with _lock:
        data = load_cache(path)
        data[key] = {"tuning": tuning, "ms": ms}
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = f"{path}.tmp{os.getpid()}"
        with open(tmp, "w") as fh:
            json.dump(data, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)


def pick(results: list[tuple[dict, float]]) -> tuple[dict, float]:
    """Fastest candidate; ties keep the earlier (default-first) one."""
    best = None
    for tuning, ms in results:
        if best is None or ms < best[1]:
            best = (tuning, ms)
    if best is None:
        raise ValueError("no candidates")
    return best


def tune(plan, x1, x2, F, f, units: str = "unit", candidates=None, reps: int = 5, use_cache: bool = True,
         path: str | None = None) -> dict:
    """Measure the candidates on plan with points (x1, x2), coefficients F and
    values f; apply the fastest to the plan, re-bin its points and return
    {"tuning": ..., "ms": ..., "cached": bool, "trials": [...]}."""
    import torch

    name = torch.cuda.get_device_name(plan.stream.device if hasattr(plan.stream, "device") else None)
    key = cache_key(plan.N1, plan.N2, plan.sigma, plan.K, x1.numel(), name)
    if use_cache:
        hit = load_cache(path).get(key)
        if hit:
            plan.set_tuning(**hit["tuning"])
            plan.set_points(x1, x2, units=units)
            return {"tuning": hit["tuning"], "ms": hit["ms"], "cached": True, "trials": []}
    trials = []
    fo = torch.empty(x1.numel(), dtype=plan.cdtype, device=x1.device)
    Fo = torch.empty(plan.N1 * plan.N2, dtype=plan.cdtype, device=x1.device)
    plan.enable_timing(True)
    for cand in candidates or _DEFAULT_CANDIDATES:
        plan.set_tuning(**cand)
        plan.set_points(x1, x2, units=units)
        best = float("inf")
        for _ in range(reps + 1):
            plan.forward(F, out=fo)
            plan.adjoint(f, out=Fo)
            t = plan.timings()
            ms = sum(t[k] for k in ("pad_ms", "fft_type2_ms", "halo_fill_ms", "gather_ms", "spread_ms", "fold_ms",
                                    "fft_type1_ms", "crop_ms"))
            best = min(best, ms)
        trials.append((dict(cand), best))
    plan.enable_timing(False)
    tuning, ms = pick(trials)
    plan.set_tuning(**tuning)
    plan.set_points(x1, x2, units=units)
    if use_cache:
        store(key, tuning, ms, path)
    return {"tuning": tuning, "ms": ms, "cached": False, "trials": trials}
