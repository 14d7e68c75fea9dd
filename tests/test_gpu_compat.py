"""A compiled C++ caller that uses only the reference's signatures
(NFFT2_2D_GPU float/double overloads, the Calculate/Destroy plan functions,
NDFT2_2D_GPU), linked against libnfft2d_gb300.so -- the drop-in path for
reference callers such as Synthesis/PSO/Synthesis.cu -- checked against the
oracle.  Tolerances: float overload vs exact NDFT rel-L2 <= 1e-5; double
overload vs the restated algorithm <= 1e-12; NDFT2_2D_GPU vs exact <= 1e-12."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    """compat_driver.cpp (next to this file) built with g++ against the
    library, as a reference caller would build its own code."""
    from miscellaneous_gb300 import build as b
    lib = b.build()
    cuda = b.cuda_home()
    exe = str(tmp_path_factory.mktemp("compat") / "nfft2d_compat_driver")
    lib_dir = os.path.dirname(lib)
    lib64 = os.path.join(cuda, "lib64")
    r = subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(HERE, "compat_driver.cpp"), "-o", exe,
                        "-I", b.INCLUDE, "-I", os.path.join(cuda, "include"), "-L", lib_dir, "-lnfft2d_gb300",
                        "-L", lib64, "-lcudart", f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{lib64}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _run_driver(exe, tmp_path, N1, N2, M, seed):
    out = tmp_path / "compat.bin"
    r = subprocess.run([exe, str(N1), str(N2), str(M), str(seed), str(out)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = out.read_bytes()
    hdr = np.frombuffer(raw[:12], dtype=np.int32)
    n1, n2, m = (int(v) for v in hdr)
    off = 12
    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a
    x = take(np.float64, m)
    y = take(np.float64, m)
    d = take(np.complex128, m)
    rf = take(np.complex64, n1 * n2).reshape(n1, n2)
    rd = take(np.complex128, n1 * n2).reshape(n1, n2)
    rn = take(np.complex128, n1 * n2).reshape(n1, n2)
    return x, y, d, rf, rd, rn


@pytest.mark.parametrize("N1,N2,M", [(32, 32, 500), (22, 22, 121), (16, 40, 1000)])
def test_reference_signatures_via_compiled_caller(orc, driver, tmp_path, N1, N2, M):
    x, y, d, rf, rd, rn = _run_driver(driver, tmp_path, N1, N2, M, seed=N1 * 1000 + M)
    exact = orc.ndft_type1(d, x, y, N1, N2, sign=-1)
    assert orc.rel_l2(rf, exact) < 1e-5
    assert orc.rel_l2(rd, orc.nfft2_2d(d, x, y, N1, N2, sign=-1)) < 1e-12
    assert orc.rel_l2(rn, exact) < 1e-12
