"""The device's exact-arithmetic building blocks, checked on the CPU.

cube_rn (the friction term's h^3) is correctly rounded; glibc's
pow(h, 3.0), which the reference calls, is not always (about 0.08 % of
arguments), which is why hydraulic parity is to rounding level rather than
bitwise.  slide_3's tests decided on float estimates never contradict the
FP64 test.  (The integer-pipe division, cube and square root are checked
against the GPU's own instructions in test_gpu_arith.py.)"""
import ctypes as C
import os
import subprocess
import tempfile
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def numlib():
    d = tempfile.mkdtemp()
    so = os.path.join(d, "numerics_check.so")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "numerics_check.c"), "-lm"], check=True)
    lib = C.CDLL(so)
    lib.cube_rn.restype = C.c_double
    lib.cube_rn.argtypes = [C.c_double]
    lib.slide_est.restype = C.c_int
    lib.slide_est.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
    lib.slide_est_check.restype = C.c_long
    lib.slide_est_check.argtypes = [C.c_long, C.c_uint, C.POINTER(C.c_long)]
    return lib


def test_cube_is_correctly_rounded(numlib):
    rng = np.random.default_rng(5)
    hs = 10.0 ** rng.uniform(-5, 1.5, 20000)
    for h in hs:
        want = float(Fraction(float(h)) ** 3)
        assert numlib.cube_rn(float(h)) == want, h


def test_glibc_pow_cube_is_not_always_correctly_rounded(numlib):
    # documents the source of the last-bit differences against the reference
    rng = np.random.default_rng(6)
    hs = 10.0 ** rng.uniform(-5, 1.5, 200000)
    libm = C.CDLL("libm.so.6")
    libm.pow.restype = C.c_double
    libm.pow.argtypes = [C.c_double, C.c_double]
    diff = sum(1 for h in hs if libm.pow(float(h), 3.0) != numlib.cube_rn(float(h)))
    assert diff < 0.01 * len(hs)


def test_slide_estimates_never_contradict_the_fp64_test(numlib):
    decided = C.c_long()
    n = 4_000_000
    assert numlib.slide_est_check(n, 7, C.byref(decided)) == 0
    # the estimates decide the tests away from the threshold
    assert decided.value > n // 3, decided.value
    special = [float("nan"), float("inf"), -float("inf"), 1e308, -1e308, 1e-310, 0.0, -0.0,
               -9999.0, 123.5]
    for e in special:
        for e2 in special:
            for w in special:
                for diag in (0, 1):
                    with np.errstate(all="ignore"):
                        d = np.float64(e) - np.float64(e2)
                        drop = d / 1.41 if diag else d
                    r = numlib.slide_est(e, e2, w, diag)
                    assert r == 2 or r == int(drop > w), (e, e2, w, diag, r)


def test_exact_sort_matches_std_sort(tmp_path):
    """The drainage order (hc_host.cpp) is std::sort's permutation, ties
    included, also when its sub-ranges are sorted by several threads."""
    root = os.path.dirname(HERE)
    exe = str(tmp_path / "sort_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-o", exe,
                    os.path.join(HERE, "sort_check.cpp"),
                    os.path.join(root, "hail-caesar_gb300", "csrc", "hc_host.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
