"""The snapshot store's division by dt (fwi_gb300/csrc/fwi_div.cuh: a
reciprocal and two fused multiply-add refinement steps instead of a full
division per cell) against CUDA's IEEE division, bit for bit, over all 2^32
values of the dividend: for the time steps of the benchmark workloads, the
divisors at the edges of a binade, and seeded random time steps."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("div") / "div_check.so")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--fmad=false",
                    "-Xcompiler", "-fPIC", "-shared", "-I", os.path.join(ROOT, "fwi_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "div_check.cu"), "-o", out], check=True)
    lb = C.CDLL(out)
    lb.div_check.argtypes = [C.c_float, C.c_float, C.POINTER(C.c_ulonglong), C.POINTER(C.c_uint)]
    return lb


def divisors():
    f = np.float32
    out = [f(1e-3), f(2e-3), f(1.5625e-3), f(2.5e-3), f(1.0), f(0.5), f(2.0 ** -10),
           np.nextafter(f(2.0 ** -9), f(0)), np.nextafter(f(1e-3), f(1)), f(3e-3), f(7e-4)]
    rng = np.random.default_rng(2024)
    out += [f(x) for x in 10.0 ** rng.uniform(-4.5, -1.0, size=16)]
    return out


@pytest.mark.parametrize("b", divisors(), ids=lambda b: f"{float(b):.9g}")
def test_division_by_dt_matches_ieee_division(lib, b):
    y = np.float32(1.0) / b  # the host reciprocal, as the library computes it
    bad, first = C.c_ulonglong(0), C.c_uint(0)
    assert lib.div_check(C.c_float(b), C.c_float(y), C.byref(bad), C.byref(first)) == 0
    assert bad.value == 0, f"{bad.value} mismatches, first dividend bits {first.value:#010x}"
