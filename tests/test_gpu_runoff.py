"""Distributed TOPMODEL rainfall-runoff (spatially_complex_rainfall: every
cell takes its own runoff, catchment_water_input_and_hydrology(flow_timestep,
runoff) LSDCatchmentModel.cpp:3544-3607, runoffGrid LSDRainfallRunoff.cpp)
on the device, against the oracle, whose restatement of this path
tests/test_oracle_pin.py pins to the live reference.

The device tabulates the runoff per rain state (every cell of a zone has the
same recurrence) and forms the two water-input sums state by state, where the
reference adds cell by cell: waterinput agrees to rounding level, the states
to the same tolerances as the other parity tests."""
import ctypes as C

import numpy as np
import pytest

import synth
from helpers import assert_bitwise, assert_close

pytestmark = pytest.mark.gpu
H_ATOL = 1e-9


def zones(p, k):
    """k rain zones in bands of rows (values 1 .. k)."""
    z = np.ones((p.imax + 2, p.jmax + 2), np.int32)
    rows = np.arange(p.imax + 2)
    for n in range(k):
        z[(rows * k) // (p.imax + 2) == n, :] = n + 1
    return z


def run_pair(case, n, oracle_mod, rf=None):
    import hc
    m = hc.Model(case, prepare=False)
    o = oracle_mod.Oracle(case)
    if rf is not None:
        m.upload("rfarea", rf)
        o.field("rfarea")[...] = rf
    m.prepare()
    g = m.run(n)
    r = o.iterate(n)
    return m, g, o, r


def check(m, g, o, r, sediment=False):
    assert g.shape == r.shape, (g.shape, r.shape)
    assert_bitwise(g[:, 0], r[:, 0], "counter")
    assert_close(g[:, [1, 2, 3, 9]], r[:, [1, 2, 3, 9]], 0, "records", rtol=1e-9)
    assert_close(g[:, 5], r[:, 5], 1e-12, "waterinput", rtol=1e-9)
    assert_close(g[:, 4], r[:, 4], 1e-12, "waterOut", rtol=1e-6)
    assert np.max(r[:, 5]) > 0, "no runoff entered the grid"
    for k in ("elev", "water_depth"):
        assert_close(m.field(k), o.field(k), H_ATOL, k)
    for k in ("qx", "qy"):
        assert_close(m.field(k), o.field(k), 1e-9, k, rtol=1e-6)
    if sediment:
        assert_bitwise(m.field("index"), o.field("index"), "index")
        for k in ("grain", "Vsusptot"):
            assert_close(m.field(k), o.field(k), H_ATOL, k)


def test_runoff_one_zone_hydro(gpu_lib, oracle_mod):
    case = synth.catchment_case(n=40, DX=20.0, hours=72, relief=60.0, hydro_only=True,
                                lateral=False, storm_start_h=0.5)
    case.params.spatially_complex_rainfall = 1
    m, g, o, r = run_pair(case, 4000, oracle_mod)
    check(m, g, o, r)


def test_runoff_three_zones_with_erosion(gpu_lib, oracle_mod):
    """Three zones: zones 1 and 2 take their rain columns, zone 3 none (the
    reference's rain grid stops before the last zone)."""
    case = synth.catchment_case(n=33, DX=20.0, hours=72, relief=60.0, lateral=False,
                                storm_start_h=0.5)
    p = case.params
    p.rfnum = 3
    rain1 = np.asarray(case.rain, np.float32)[:, :1]
    case.rain = np.ascontiguousarray(np.hstack([rain1, 0.5 * rain1, 2.0 * rain1]))
    p.spatially_complex_rainfall = 1
    m, g, o, r = run_pair(case, 1500, oracle_mod, rf=zones(p, 3))
    check(m, g, o, r, sediment=True)


def test_runoff_adjoint_rejected(gpu_lib):
    import hc
    case = synth.catchment_case(n=24, DX=20.0, hours=12, relief=40.0, hydro_only=True,
                                lateral=False)
    case.params.spatially_complex_rainfall = 1
    m = hc.Model(case)
    rec = np.zeros((4, 22))
    st = m.lib.hc_adj_forward(m.h, 4, None, rec.ctypes.data, None, 0, C.byref(C.c_int64()))
    assert hc.STATUS.get(st) == "HC_ERR_UNSUPPORTED", st
