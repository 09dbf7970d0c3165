"""The member-level entry points (the member-by-member drop-in path): a state
computed by the oracle is uploaded field by field in the reference's layout,
one member is called on the GPU and the same member on the oracle, and the
results are compared.  This exercises hc_upload/hc_download layout
conversions and hc_set_scalars as a C++ caller would use them."""
import numpy as np
import pytest

import synth
from hc_abi import hc_scalars
from helpers import assert_bitwise, assert_close

pytestmark = pytest.mark.gpu

FIELDS = ["elev", "water_depth", "qx", "qy", "qxs", "qys", "Vsusptot", "Vel", "Tau", "bedrock",
          "spat_var_mannings", "area", "index", "down_scan", "edge", "vel_dir", "rfarea"]
SED = ["ss", "sr", "sl", "su", "sd", "grain", "strata"]


def mid_run(oracle_mod, case, n):
    import hc
    o = oracle_mod.Oracle(case)
    o.iterate(n)
    m = hc.Model(case, prepare=False)
    names = FIELDS + ([] if case.params.hydro_only else SED)
    for k in names:
        m.upload(k, o.field(k))
    s = hc_scalars()
    for k in ("cycle", "time_step", "maxdepth", "waterinput", "waterOut", "counter", "erode_call",
              "erode_mult", "lateralcounter", "time_1", "baseflow", "grain_array_tot", "sediQ",
              "globalsediq"):
        setattr(s, k, o.scalar(k))
    m.set_scalars(s)
    return o, m


@pytest.fixture(scope="module")
def erosion_case():
    return synth.catchment_case(n=33, DX=20.0, hours=72, relief=60.0, lateral=True)


def test_flow_route_and_depth_update(gpu_lib, oracle_mod, erosion_case):
    o, m = mid_run(oracle_mod, erosion_case, 700)
    m.flow_route()
    o.lib.hco_flow_route(o.h)
    for k in ("qx", "qy", "qxs", "qys", "vel_dir"):
        assert_close(m.field(k), o.field(k), 1e-12, k, rtol=1e-12)
    m.depth_update()
    o.lib.hco_depth_update(o.h)
    assert_close(m.field("water_depth"), o.field("water_depth"), 1e-12, "water_depth")
    assert abs(m.scalars().maxdepth - o.scalar("maxdepth")) <= 1e-12


def test_scan_area_and_flux_out(gpu_lib, oracle_mod, erosion_case):
    o, m = mid_run(oracle_mod, erosion_case, 500)
    m.scan_area()
    o.lib.hco_scan_area(o.h)
    assert_bitwise(m.field("down_scan"), o.field("down_scan"), "down_scan")
    m.water_flux_out()
    o.lib.hco_water_flux_out(o.h)
    assert_bitwise(m.field("water_depth"), o.field("water_depth"), "water_depth")
    assert_close(m.scalars().waterOut, o.scalar("waterOut"), 0, "waterOut", rtol=1e-12)


def test_erode_member(gpu_lib, oracle_mod, erosion_case):
    o, m = mid_run(oracle_mod, erosion_case, 900)
    t_gpu = m.erode(2.0)
    t_cpu = o.lib.hco_erode(o.h, 2.0)
    assert_close(t_gpu, t_cpu, 0, "tempbmax", rtol=1e-9)
    assert_bitwise(m.field("index"), o.field("index"), "index")
    for k in ("elev", "grain", "strata", "Vsusptot", "Tau", "Vel", "ss", "sr", "su"):
        assert_close(m.field(k), o.field(k), 1e-10, k, rtol=1e-9)
    assert_close(m.scalars().time_step, o.scalar("time_step"), 0, "time_step", rtol=1e-12)


@pytest.mark.parametrize("n", [33, 96])
def test_in_channel_landsliding_member(gpu_lib, oracle_mod, n):
    """A mid-run state whose wet cells (the only ones slide_3 tests) are
    raised by 25 m at one in six, the same in the oracle and on the device:
    slides follow one another within columns and across them, so re-tests
    queue behind later flagged positions and batches are cut short by
    moves."""
    case = synth.catchment_case(n=n, DX=10.0, hours=72, relief=60.0, lateral=False,
                                storm_start_h=0.5)
    o, m = mid_run(oracle_mod, case, 900)
    e = o.field("elev")
    wet = np.argwhere(o.field("water_depth") > 0)
    rng = np.random.default_rng(3)
    pick = wet[rng.choice(len(wet), size=len(wet) // 6, replace=False)]
    e[pick[:, 0], pick[:, 1]] += 25.0
    m.upload("elev", e)
    before = np.array(e, copy=True)
    m.in_channel_landsliding()
    o.lib.hco_in_channel_landsliding(o.h)
    assert np.sum(o.field("elev") != before) > 100, "too few moves to test the replay"
    assert_bitwise(m.field("elev"), o.field("elev"), "elev")
    assert_bitwise(m.field("index"), o.field("index"), "index")
    assert_close(m.field("grain"), o.field("grain"), 1e-12, "grain", rtol=1e-12)


def test_lateral_member(gpu_lib, oracle_mod, erosion_case):
    o, m = mid_run(oracle_mod, erosion_case, 1200)
    m.lateral_channel_erode()
    o.lib.hco_lateral_channel_erode(o.h)
    assert_close(m.field("edge"), o.field("edge"), 1e-12, "edge", rtol=1e-9)
