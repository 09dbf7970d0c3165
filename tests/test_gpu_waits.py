"""The bounded device waits: the drainage recomputation's cooperative kernel
waits at grid barriers, and every wait gives up after a bounded number of
spins.  hc_test_bounded_waits shortens the bound and makes the barrier
expect one block more than was launched, so the wait runs out without any
fault: hc_run returns HC_ERR_TIMEOUT, the context stays usable, and the next
hc_run makes the recomputation again and goes on exactly as a run that never
timed out."""
import pytest

import synth
from helpers import assert_bitwise

pytestmark = pytest.mark.gpu


def test_drainage_wait_runs_out_then_run_resumes(gpu_lib):
    import hc
    # erosion on: the elevations change, so every baseflow change sweeps
    # the drainage area again (a hydro-only run computes it once)
    case = synth.catchment_case(n=48, DX=20.0, hours=72, relief=60.0, hydro_only=False,
                                lateral=False, storm_start_h=0.5)
    ref = hc.Model(case)
    ra = ref.run(1500)
    assert ref.run_stats()["drainage"][0] >= 1, "no baseflow change in the window"
    m = hc.Model(case)
    m.test_bounded_waits(1 << 12, 1)
    with pytest.raises(hc.HCError, match="HC_ERR_TIMEOUT"):
        m.run(1500)
    k = int(m.scalars().counter)
    assert 0 < k < 1500
    # the context answers, and with the normal bounds the run goes on from
    # the redone recomputation as if nothing had happened
    m.test_bounded_waits(0, 0)
    rb = m.run(1500 - k)
    assert_bitwise(rb, ra[k:], "records")
    for f in ("water_depth", "qx", "qy", "area", "down_scan", "elev", "index"):
        assert_bitwise(m.field(f), ref.field(f), f)
