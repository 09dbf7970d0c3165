"""The integer-pipe IEEE division of the kernels (ddiv_rn in
hc_internal.cuh) against the hardware's division, bit for bit (and the
cube, square root and float conversions likewise): 2^30
quotients per input family (arbitrary bit patterns, normal operands, edge
significands, near-integer quotients, edges of the normal range, the
model's magnitudes, signed zero and subnormal dividends); and the
throughput of both, printed."""
import ctypes as C
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FAMILIES = ["bit patterns", "normal", "edge significands", "near-integer quotients",
            "range edges", "model magnitudes", "zero and subnormal dividends"]


@pytest.fixture(scope="module")
def arith(tmp_path_factory):
    import build as hcbuild
    so = str(tmp_path_factory.mktemp("arith") / "arith_check.so")
    cmd = [hcbuild.nvcc()] + hcbuild.ARCH + hcbuild.NVFLAGS + \
        ["-shared", "-o", so, os.path.join(HERE, "arith_check.cu")]
    subprocess.run(cmd, check=True, capture_output=True)
    lib = C.CDLL(so)
    lib.arith_check.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.POINTER(C.c_uint64),
                                C.POINTER(C.c_double)]
    lib.arith_check_prepared.argtypes = [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64),
                                         C.POINTER(C.c_double)]
    lib.arith_check_cube.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_double)]
    lib.arith_check_conv.argtypes = [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_double)]
    lib.arith_check_sqrt.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_double)]
    lib.arith_time.argtypes = [C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    return lib


@pytest.mark.parametrize("mode", range(len(FAMILIES)), ids=FAMILIES)
def test_division_matches_hardware(arith, mode):
    bad = C.c_uint64(0)
    first = (C.c_double * 4)()
    assert arith.arith_check(1 << 30, 1 + mode, mode, C.byref(bad), first) == 0
    assert bad.value == 0, "%d mismatches; first a=%r b=%r got %r want %r" % (
        bad.value, first[0], first[1], first[2], first[3])


def test_division_by_prepared_divisors(arith):
    """Divisors prepared on the host (exact reciprocal), as DX and the
    Einstein constants are."""
    bad = C.c_uint64(0)
    first = (C.c_double * 4)()
    assert arith.arith_check_prepared(1 << 30, 99, C.byref(bad), first) == 0
    assert bad.value == 0, "%d mismatches; first a=%r b=%r got %r want %r" % (
        bad.value, first[0], first[1], first[2], first[3])


@pytest.mark.parametrize("mode", range(3), ids=["bit patterns", "depths", "short significands"])
def test_cube_on_integer_pipe(arith, mode):
    """icube_rn (the friction term's h^3 on the integer pipe) against the
    FP64 cube_rn over 2^30 arguments; where they differ, the exact cube
    decides, and it must be icube_rn's."""
    from fractions import Fraction
    import math
    bad = C.c_uint64(0)
    keep = (C.c_double * (3 * 64))()
    assert arith.arith_check_cube(1 << 30, 7 + mode, mode, C.byref(bad), keep) == 0
    for i in range(min(64, bad.value)):
        h, x, y = keep[3 * i], keep[3 * i + 1], keep[3 * i + 2]
        exact = Fraction(h) ** 3
        want = float(exact) if abs(exact) < Fraction(2) ** 1023 else math.copysign(math.inf, h)
        assert x == want, "h=%r: icube %r, cube_rn %r, exact %r" % (h, x, y, want)


@pytest.mark.parametrize("mode", range(3), ids=["bit patterns", "positive normal", "squares"])
def test_sqrt_on_integer_pipe(arith, mode):
    """isqrt_rn (the Froude limiter's and the flow velocity's square roots)
    against the hardware square root, 2^30 arguments per family."""
    bad = C.c_uint64(0)
    first = (C.c_double * 4)()
    assert arith.arith_check_sqrt(1 << 30, 11 + mode, mode, C.byref(bad), first) == 0
    assert bad.value == 0, "%d mismatches; first x=%r got %r want %r" % (
        bad.value, first[0], first[1], first[2])


def test_float_conversions_on_integer_pipe(arith):
    """d2f_i / f2d_i (the edge output's float sums) against the conversion
    instructions, over 2^30 values each."""
    bad = C.c_uint64(0)
    first = (C.c_double * 4)()
    assert arith.arith_check_conv(1 << 30, 5, C.byref(bad), first) == 0
    assert bad.value == 0, "%d mismatches; first x=%r f=%r" % (bad.value, first[0], first[1])


def test_division_throughput(arith):
    tn, ti = C.c_float(0), C.c_float(0)
    assert arith.arith_time(2000, C.byref(tn), C.byref(ti)) == 0
    print("divisions: hardware %.3f ms, integer pipe %.3f ms (%.2fx)" %
          (tn.value, ti.value, tn.value / ti.value))
