"""Build recipe for libnfft2d_gb300.so (sm_103a).

Each CUDA translation unit is compiled by nvcc in parallel, then linked into
one shared library in ``miscellaneous_gb300/lib``.  Objects are rebuilt only
when a source or header is newer than the object.  No cmake, no setuptools.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ_DIR = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB_NAME = "libnfft2d_gb300.so"
LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: host arithmetic rounds as written on every host (the Arm
# host compiler would otherwise fuse multiply-adds), so host-side sizes and
# axes match an IEEE restatement bit for bit.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnfft2d_gb300.so")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _headers() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
                  + glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.cuh")))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose_ptxas: bool) -> tuple[str, str]:
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _headers()) and not verbose_ptxas:
        return obj, ""
    tmp = obj + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH_FLAGS, *NVCC_FLAGS, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", tmp]
    if verbose_ptxas:
        cmd[1:1] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, obj)
    return obj, r.stderr


def build(verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    """Compile every .cu under csrc/ for sm_103a and link libnfft2d_gb300.so."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = jobs or min(len(sources), os.cpu_count() or 4)
    objs, logs = [], []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for obj, log in ex.map(lambda s: _compile(s, verbose_ptxas), sources):
            objs.append(obj)
            if log:
                logs.append(log)
    if verbose_ptxas:
        sys.stderr.write("".join(logs))
    if _stale(LIB_PATH, objs):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        lib64 = os.path.join(cuda_home(), "lib64")
        cmd = [nvcc(), *ARCH_FLAGS, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp,
               "-L", lib64, "-lcufft", "-lcudart", "-Xlinker", "-rpath", "-Xlinker", lib64]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
