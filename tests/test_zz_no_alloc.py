"""hc_depth_update_noalloc: depth_update on caller-owned device buffers with
its working memory in a fixed array of the library, against hc_depth_update
(the context's entry point) on the same state, for two calls in a row.

The file is named to be collected last, so that it also runs after every
other test has used the library in the same process."""
import ctypes as C

import numpy as np
import pytest

import synth

HC_ERR_ARG = 1
MAX_COLS = 16383  # HC_DEPTH_NOALLOC_MAX_COLS


def declare(lib):
    f = lib.hc_depth_update_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double] + [C.c_void_p] * 10 + \
        [C.c_char_p, C.c_size_t]
    return f


def test_rejects_grids_wider_than_the_scratch(gpu_lib):
    f = declare(gpu_lib)
    err = C.create_string_buffer(256)
    fake = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = f(10, MAX_COLS + 1, 10.0, 1.0, *([fake] * 10), err, 256)
    assert st == HC_ERR_ARG
    assert b"HC_DEPTH_NOALLOC_MAX_COLS" in err.value, err.value


@pytest.mark.gpu
def test_noalloc_matches_depth_update_twice(gpu_lib):
    import torch
    import hc
    f = declare(gpu_lib)
    case = synth.catchment_case(n=33, DX=20.0, hours=72, relief=60.0, lateral=False,
                                storm_start_h=0.1)
    p = case.params
    m = hc.Model(case)
    m.run(600, records=False)
    dev = {k: torch.from_numpy(np.ascontiguousarray(m.field(k))).cuda()
           for k in ("down_scan", "elev", "qx", "qy", "qxs", "qys", "water_depth", "Vsusptot")}
    assert dev["down_scan"].dtype == torch.int32
    maxd = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    err = C.create_string_buffer(256)
    for call in range(2):
        m.depth_update()
        s = m.scalars()
        ptr = [C.c_void_p(dev[k].data_ptr()) for k in
               ("down_scan", "elev", "qx", "qy", "qxs", "qys", "water_depth", "Vsusptot")]
        st = f(p.imax, p.jmax, p.DX, s.flow_timestep, *ptr, C.c_void_p(maxd.data_ptr()),
               C.c_void_p(stream.cuda_stream), err, 256)
        assert st == 0, err.value
        torch.cuda.synchronize()
        h_ref = m.field("water_depth")
        assert s.maxdepth > 0
        # both compute the same IEEE quotients in the same order: bit for bit
        for k in ("water_depth", "Vsusptot"):
            got = dev[k].cpu().numpy()
            ref = m.field(k)
            assert np.array_equal(got, ref, equal_nan=True), (call, k, np.nanmax(np.abs(got - ref)))
        assert maxd.item() == s.maxdepth, (call, maxd.item(), s.maxdepth)
        assert np.abs(h_ref).max() > 0
