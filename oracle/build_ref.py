"""Build recipe for oracle/_ref: the reference's own GPU spreading as a parity
oracle.  TEST INFRASTRUCTURE ONLY.

Two artefacts, both written only into ``oracle/_ref/`` (git-ignored):

* ``nfft2_2d_ref.cubin`` -- ``NFFT/NFFT2_2D.cu`` compiled unchanged from the
  reference checkout (``REFERENCE_ROOT``, default ``/root/reference``) for
  sm_103a with relocatable device code (its interpolation kernel launches a
  child grid per point), with the stand-in headers of ``oracle/ref_shims``
  for the four headers the reference does not ship, then device-linked with
  the CUDA device runtime (``libcudadevrt.a``) by ``nvlink``.  A cubin holds
  device code only, so it is built where the reference sources are and
  travels as it is; it is rebuilt only when the reference file is present.
* ``libref_harness.so`` -- ``oracle/ref_harness.cpp`` (the restated host side
  of ``NFFT2_2D_GPU``, loading the cubin with the driver API), compiled by g++
  on whatever machine runs the tests.

Run ``python -m oracle.build_ref`` or call ``build()``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SHIMS = os.path.join(HERE, "ref_shims")
HARNESS_SRC = os.path.join(HERE, "ref_harness.cpp")
CUBIN = os.path.join(REF_DIR, "nfft2_2d_ref.cubin")
HARNESS_LIB = os.path.join(REF_DIR, "libref_harness.so")


def reference_root() -> str:
    return os.environ.get("REFERENCE_ROOT", "/root/reference")


def _nvcc() -> str | None:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def _cuda_home() -> str | None:
    nv = _nvcc()
    return os.path.dirname(os.path.dirname(os.path.realpath(nv))) if nv else None


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_cubin(force: bool = False) -> str | None:
    """Compile and device-link the reference's NFFT2_2D.cu; None when the
    reference checkout is absent (the GPU machine uses the cubin built here)."""
    src = os.path.join(reference_root(), "NFFT", "NFFT2_2D.cu")
    if not os.path.exists(src):
        return CUBIN if os.path.exists(CUBIN) else None
    shims = [os.path.join(SHIMS, f) for f in sorted(os.listdir(SHIMS))]
    if not force and not _stale(CUBIN, [src, os.path.join(os.path.dirname(src), "NFFT2_2D.cuh")] + shims):
        return CUBIN
    nvcc = _nvcc()
    if nvcc is None:
        raise RuntimeError("nvcc not found")
    cuda = _cuda_home()
    os.makedirs(REF_DIR, exist_ok=True)
    rdc = os.path.join(REF_DIR, "nfft2_2d_ref_rdc.cubin")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-rdc=true", "-cubin",
                    "-I", SHIMS, "-I", os.path.dirname(src), src, "-o", rdc], check=True)
    nvlink = os.path.join(os.path.dirname(nvcc), "nvlink")
    tmp = CUBIN + f".tmp{os.getpid()}"
    subprocess.run([nvlink, "-arch=sm_103a", rdc, "-L", os.path.join(cuda, "lib64"), "-lcudadevrt", "-o", tmp],
                   check=True)
    os.replace(tmp, CUBIN)
    os.remove(rdc)
    return CUBIN


def build_harness(force: bool = False) -> str:
    """Compile the host-side harness against the CUDA runtime, driver and cuFFT."""
    if not force and not _stale(HARNESS_LIB, [HARNESS_SRC]):
        return HARNESS_LIB
    cuda = _cuda_home()
    if cuda is None:
        raise RuntimeError("CUDA toolkit not found")
    os.makedirs(REF_DIR, exist_ok=True)
    lib64 = os.path.join(cuda, "lib64")
    tmp = HARNESS_LIB + f".tmp{os.getpid()}"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", HARNESS_SRC, "-o", tmp,
                    "-I", os.path.join(cuda, "include"), "-L", lib64, "-L", os.path.join(lib64, "stubs"),
                    "-lcufft", "-lcudart", "-lcuda", f"-Wl,-rpath,{lib64}"], check=True)
    os.replace(tmp, HARNESS_LIB)
    return HARNESS_LIB


def build(force: bool = False) -> tuple[str | None, str]:
    return build_cubin(force), build_harness(force)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
