"""Hillslope processes on the device against the oracle: global landsliding
(global_landsliding, LSDCatchmentModel.cpp:5529-5654: sweeps over every cell
until nothing moves) and creep (creep :5293-5427), as member calls on a DEM
with a raised block steeper than the failure angle, and inside hc_run, where
the block is raised again in mid-run so that the daily sweep and the 10-day
creep move material after the first iteration."""
import numpy as np
import pytest

import synth
from hc_abi import STEP_FIELDS
from helpers import assert_bitwise, assert_close

pytestmark = pytest.mark.gpu

COL = {k: i for i, k in enumerate(STEP_FIELDS)}


def raised_case(hours=72):
    """A dry 64 x 64 catchment (no rain: the time step stays long, so the
    run reaches the daily and two-day intervals quickly) with an 80 m block;
    creep every two simulated days instead of ten."""
    case = synth.catchment_case(n=64, DX=20.0, hours=hours, relief=60.0, lateral=False,
                                storm_start_h=10000.0)
    case.rain[:] = 0
    case.params.creep_time_interval = 2880
    z = case.elev.copy()
    z[20:30, 24:34] += 80.0  # 80 m cliffs: far past tan(45 deg) * DX = 20 m
    case.elev = np.ascontiguousarray(z)
    return case


def test_global_landsliding_member(gpu_lib, oracle_mod):
    import hc
    case = raised_case()
    m = hc.Model(case)
    o = oracle_mod.Oracle(case)
    o.prepare()
    e0 = m.field("elev")
    sweeps = m.global_landsliding()
    o.lib.hco_global_landsliding(o.h)
    assert sweeps > 1
    moved = np.sum(m.field("elev") != e0)
    assert moved > 50, moved
    # the same tests and moves in the same order: bit for bit
    assert_bitwise(m.field("elev"), o.field("elev"), "elev")
    # 80 m cliffs need more than the 200 sweeps one call makes (each move is
    # capped at ERODEFACTOR): a second call goes on from there, as the
    # reference's next daily call would
    m.global_landsliding()
    o.lib.hco_global_landsliding(o.h)
    assert_bitwise(m.field("elev"), o.field("elev"), "elev after a second call")


def test_creep_member(gpu_lib, oracle_mod):
    import hc
    case = raised_case()
    m = hc.Model(case)
    o = oracle_mod.Oracle(case)
    o.prepare()
    e0 = m.field("elev")
    m.creep(0.028)
    o.lib.hco_creep(o.h, 0.028)
    assert np.sum(m.field("elev") != e0) > 100
    assert_bitwise(m.field("elev"), o.field("elev"), "elev")


def test_hillslope_in_run_after_first_iteration(gpu_lib, oracle_mod):
    """hc_run for 72 simulated hours: creep and global landsliding at
    iteration 1, a second block raised after 400 iterations, then the daily
    sweeps and the creep of day 2 inside the run."""
    import hc
    case = raised_case(hours=72)
    m = hc.Model(case)
    o = oracle_mod.Oracle(case)
    g1 = m.run(400)
    r1 = o.iterate(400)
    assert_bitwise(m.field("elev"), o.field("elev"), "elev after 400")
    z = m.field("elev")
    z[30:36, 40:46] += 60.0
    m.upload("elev", z)
    o.field("elev")[...] = z
    before = z.copy()
    g2 = m.run(30000)
    r2 = o.iterate(-1)
    g = np.concatenate([g1, g2])
    r = np.concatenate([r1, r2])
    assert g.shape == r.shape
    assert g[-1, COL["cycle"]] > 2880, "the run did not reach the second creep"
    assert_close(g[:, COL["cycle"]], r[:, COL["cycle"]], 0, "cycle", rtol=1e-9)
    after = m.field("elev")
    assert np.sum(after[28:38, 38:48] != before[28:38, 38:48]) > 20, "no move after iteration 1"
    assert_close(after, o.field("elev"), 1e-9, "elev")
    stats = m.run_stats()
    assert stats["global_slide"][0] >= 3 and stats["creep"][0] >= 2, stats


def test_global_landsliding_dense_wavefront(gpu_lib, oracle_mod):
    """A raw fractal DEM (pits not filled, steep at 10 m cells), where most
    cells move in the first sweeps: the device takes its wavefront sweep
    there, and the elevations are still the serial sweep's, bit for bit."""
    import hc
    case = synth.ensemble_member(3, fill=False, side_min=120, side_max=200)
    m = hc.Model(case)
    o = oracle_mod.Oracle(case)
    o.prepare()
    e0 = m.field("elev")
    m.global_landsliding()
    o.lib.hco_global_landsliding(o.h)
    changed = np.sum(m.field("elev") != e0)
    assert changed > 0.5 * case.cells, changed
    assert_bitwise(m.field("elev"), o.field("elev"), "elev")
