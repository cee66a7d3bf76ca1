"""The FP64 step's arithmetic shortcuts against the operations they stand
for, on large random samples (tests/cuda/arith_check.cu, built here with nvcc):

  * mat::dvd_known(a, b, RN(1/b)) (Markstein's correction applied twice) for
    the divisors the material laws divide by (3, the shear modulus, the time
    step, the grain density and diameter, and random ones): bit-identical to
    IEEE division (__ddiv_rn) over normal operands spanning 2^-60..2^60;
  * mat::exp_small(x), the Taylor polynomial the volume update uses for
    |x| < 2^-9: within one ulp of CUDA's exp().
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def arith(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("arith") / "libarith_check.so")
    src = os.path.join(ROOT, "tests", "cuda", "arith_check.cu")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-shared",
                    "-Xcompiler", "-fPIC", "-o", out, src], check=True, capture_output=True)
    lib = C.CDLL(out)
    lib.check_division.argtypes = [C.c_double, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_ulonglong),
                                   C.POINTER(C.c_double)]
    lib.check_exp.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_double)]
    return lib


G = 1e6 / (2.0 * (1.0 + 0.3))


@pytest.mark.parametrize("b", [3.0, G, 1e6 / (3.0 * (1.0 - 0.6)), 2e-6, 1e-5, 3e-6, 2450.0, 5.3e-4, 0.005])
def test_known_divisor_equals_ieee_division(arith, b):
    bad = C.c_ulonglong()
    ex = (C.c_double * 3)()
    assert arith.check_division(b, 1 << 26, 12345, C.byref(bad), ex) == 0
    assert bad.value == 0, (b, bad.value, list(ex))


def test_known_divisor_random_divisors(arith):
    rng = np.random.default_rng(7)
    for b in np.exp(rng.uniform(np.log(1e-9), np.log(1e9), 24)) * rng.choice([-1, 1], 24):
        bad = C.c_ulonglong()
        ex = (C.c_double * 3)()
        assert arith.check_division(float(b), 1 << 22, 99, C.byref(bad), ex) == 0
        assert bad.value == 0, (b, bad.value, list(ex))


def test_small_argument_exp_within_one_ulp(arith):
    worst = C.c_double()
    assert arith.check_exp(1 << 26, 5, C.byref(worst)) == 0
    assert worst.value <= 1.0, worst.value
