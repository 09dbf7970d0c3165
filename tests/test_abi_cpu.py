"""C ABI checks that need no GPU: the library loads, exports every entry
point include/hc_gpu.h declares, and its parameter defaults and field sizes
agree with the Python mirror (hail-caesar_gb300/hc_abi.py)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import hc_abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "hc_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:[\w\s\*]+?)\b(hc_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("hc_create", "hc_destroy", "hc_upload", "hc_download", "hc_flow_route",
                 "hc_depth_update", "hc_scan_area", "hc_water_flux_out", "hc_erode",
                 "hc_lateral_channel_erode", "hc_in_channel_landsliding", "hc_run"):
        assert must in names


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = C.CDLL(os.path.join(ROOT, "hail-caesar_gb300", "libhc_gpu.so"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_params_default_matches_python(gpu_lib):
    p = hc_abi.hc_params()
    gpu_lib.hc_params_default(C.byref(p), 50, 70, 12.5)
    q = hc_abi.default_params(50, 70, 12.5)
    assert hc_abi.params_to_dict(p) == hc_abi.params_to_dict(q)


def test_struct_sizes_match_header_layout():
    # hc_params is all int32/double members; its size must be a multiple of 8
    assert C.sizeof(hc_abi.hc_params) % 8 == 0
    assert C.sizeof(hc_abi.hc_step_record) == 14 * 8
    assert C.sizeof(hc_abi.hc_mass) == 6 * 8


@pytest.mark.parametrize("name", hc_abi.FIELDS)
def test_field_counts_match_reference_layout(gpu_lib, name):
    p = hc_abi.default_params(7, 11, 10.0)
    n = gpu_lib.hc_field_count(C.byref(p), hc_abi.FIELD_ID[name])
    es = gpu_lib.hc_field_elsize(hc_abi.FIELD_ID[name])
    shape = hc_abi.field_shape(p, name)
    assert n == int(np.prod(shape))
    assert es == np.dtype(hc_abi.field_dtype(name)).itemsize


def test_create_rejects_bad_arguments(gpu_lib):
    h = C.c_void_p()
    p = hc_abi.default_params(2, 2, 10.0)  # too small
    assert gpu_lib.hc_create(C.byref(p), 0, C.byref(h)) == 1
    p = hc_abi.default_params(10, 10, -1.0)
    assert gpu_lib.hc_create(C.byref(p), 0, C.byref(h)) == 1
    p = hc_abi.default_params(10, 10, 10.0)
    p.vegetation_on = 1
    assert gpu_lib.hc_create(C.byref(p), 0, C.byref(h)) == 7  # unsupported
    assert gpu_lib.hc_create(None, 0, C.byref(h)) == 1
