"""Pins the oracle (oracle/hc_oracle.cpp, the CPU restatement) to the
reference:

* the reference's own known-good answers (test/basic_kga_tests.py): the
  Boscastle 50 m water-depth raster at 3360 min and the 72 h hydrograph,
  normal and flipped left-right, with the reference test's rtol = 1e-3;
* committed fixtures made by the unmodified reference sources on seeded
  synthetic cases (tests/golden/make_golden.py): bit-identical state;
* the live reference harness, where it has been built here.
"""
import json
import os

import numpy as np
import pytest

import synth
from hc_abi import params_from_dict
from helpers import assert_bitwise

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def boscastle_case(tag):
    z = np.load(os.path.join(GOLD, "boscastle_kga.npz"))
    p = params_from_dict(json.loads(str(z[tag + "_params"])))
    return synth.Case("boscastle_" + tag, p, z[tag + "_elev"], z["rain"]), z


def hydrograph(records, interval):
    """Qw column of the reference's time-series writer output_data
    (LSDCatchmentModel.cpp:2310-2478), from the per-iteration records."""
    cyc = records[:, 1]
    tot = records[:, 4]
    prev = np.concatenate([[0.0], cyc[:-1]])
    tx = interval
    newvol = oldvol = lastvol = 0.0
    rows = []
    for k in range(len(cyc)):
        cycle, previous, temptotal = cyc[k], prev[k], tot[k]
        newvol += temptotal * ((cycle - previous) * 60)
        if (np.fmod(cycle, interval) < np.fmod(previous, interval)) or (cycle - previous >= interval):
            while tx > previous and cycle >= tx:
                overvol = temptotal * ((cycle - tx) * 60)
                stepvol = newvol - oldvol
                hourvol = stepvol - overvol + lastvol
                rows.append(hourvol / (60 * interval))
                if cycle >= tx + interval:
                    lastvol = 0
                    oldvol = newvol - overvol
                if cycle < tx + interval:
                    lastvol = overvol
                    oldvol = newvol
                tx = tx + interval
    return np.array(rows)


def run_until_save(o, target, raster_interval):
    """Iterates like main.cpp until save_raster_output writes the raster
    named `target` (cycle >= save_time, save_time += interval)."""
    save_time = 0.0
    recs = []
    while True:
        r = o.iterate(1)
        recs.append(r[0])
        cycle = r[0][1]
        if cycle >= save_time:
            if int(cycle) == target:
                return np.array(recs)
            save_time += raster_interval
        assert cycle < target + 10, "passed the save point"


@pytest.mark.parametrize("tag", ["normal", "flipped"])
def test_boscastle_kga(oracle_mod, tag):
    case, z = boscastle_case(tag)
    o = oracle_mod.Oracle(case)
    recs = run_until_save(o, 3360, float(z[tag + "_raster_interval"]))
    wd = o.field("water_depth")[1:-1, 1:-1]
    got = np.array([float("%.6g" % v) for v in wd.ravel()]).reshape(wd.shape)
    np.testing.assert_allclose(got, z[tag + "_wd3360"], rtol=1e-3)
    rest = o.iterate(-1)
    q = hydrograph(np.concatenate([recs, rest]), float(z[tag + "_interval"]))
    want = z[tag + "_hydrograph"]
    assert len(q) == len(want)
    np.testing.assert_allclose(np.round(q, 6), want, rtol=1e-3)


def golden_names():
    return sorted(f[4:-4] for f in os.listdir(GOLD) if f.startswith("ref_") and f.endswith(".npz"))


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference_fixture(oracle_mod, name):
    import make_golden
    case, n = make_golden.golden_cases()[name]
    z = np.load(os.path.join(GOLD, "ref_%s.npz" % name))
    o = oracle_mod.Oracle(case)
    rec = o.iterate(n)
    assert_bitwise(rec[:, :10], z["records"], "records")
    for k in z.files:
        if k in ("records", "iterations") or k.startswith("s_"):
            continue
        got = o.field(k)
        if k in ("grain", "strata"):
            got = got[: z[k].shape[0]]
        assert_bitwise(got, z[k], k)
    for s in ("cycle", "time_step", "grain_array_tot", "sediQ", "globalsediq", "baseflow",
              "totalinputpoints", "erode_mult", "erode_call"):
        assert o.scalar(s) == float(z["s_" + s]), s


def _have_ref(oracle_mod):
    return os.path.exists(oracle_mod.REF_HARNESS)


@pytest.mark.parametrize("kind", ["reach", "catchment", "runoff"])
def test_oracle_matches_live_reference(oracle_mod, kind):
    if not _have_ref(oracle_mod):
        pytest.skip("reference harness not built (no reference checkout)")
    if kind == "reach":
        case = synth.reach_case(imax=48, jmax=20, DX=10.0, hours=24, seed=11)
        n = 3000
    elif kind == "runoff":
        # distributed TOPMODEL: every cell takes its own runoff
        case = synth.catchment_case(n=30, DX=20.0, hours=72, relief=80.0, seed=13,
                                    lateral=False, storm_start_h=0.5)
        case.params.spatially_complex_rainfall = 1
        n = 6000
    else:
        case = synth.catchment_case(n=30, DX=20.0, hours=72, relief=80.0, seed=12, lateral=True)
        n = 15000
    st, rec = oracle_mod.run_reference(case, n)
    o = oracle_mod.Oracle(case)
    r = o.iterate(n)
    assert_bitwise(r[:, :10], rec, "records")
    for k in ("elev", "water_depth", "qx", "qy", "index", "grain", "strata", "edge", "Vsusptot"):
        if k in st:
            assert_bitwise(o.field(k), st[k], k)


def test_oracle_stops_at_the_end_of_the_run(oracle_mod):
    """The main loop ends at maxcycle (:1838): once it has, iterate runs
    nothing, as hc_run returns no iterations; the grain arrays keep the
    reference's N2/LIMIT rows and a run that would need more raises instead
    of writing past them."""
    case = synth.reach_case(imax=40, jmax=16, DX=10.0, hours=1)
    o = oracle_mod.Oracle(case)
    rec = o.iterate(-1)
    assert len(rec) > 0 and rec[-1][1] / 60 >= case.params.maxcycle
    assert len(o.iterate(1)) == 0
    assert len(o.iterate(50)) == 0
    assert o.scalar("grain_full") == 0


def test_oracle_refuses_to_overflow_the_grain_rows(oracle_mod):
    """A run asking for more grain records than the N2/LIMIT rows the
    reference allocates stops with an error (the reference's arrays would
    be overrun) instead of writing past them."""
    case = synth.reach_case(imax=40, jmax=16, DX=10.0, hours=2)
    p = case.params
    p.LIMIT = (p.imax + 2) * (p.jmax + 2) // 4  # four rows
    o = oracle_mod.Oracle(case)
    with pytest.raises(RuntimeError, match="grain records"):
        o.iterate(-1)
    assert o.scalar("grain_full") == 1
