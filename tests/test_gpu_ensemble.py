"""hc_run_ensemble: several independent catchments advanced together, each
on its own stream.  Every member must end bit-identical to the same model run
alone with hc_run (the device work is deterministic), whatever the members'
sizes, parameters and pause points."""
import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu

CHECK = ["elev", "water_depth", "qx", "qy", "index", "down_scan", "grain", "Vsusptot"]


def members():
    return [
        synth.catchment_case(n=33, DX=20.0, hours=72, relief=60.0, lateral=True, seed=1,
                             storm_start_h=0.2),
        synth.catchment_case(n=41, DX=10.0, hours=72, relief=120.0, lateral=False, seed=2,
                             storm_start_h=0.2),
        synth.reach_case(imax=60, jmax=24, DX=10.0, hours=24),
        synth.catchment_case(n=24, DX=20.0, hours=72, relief=60.0, lateral=False,
                             hydro_only=True, seed=3),
    ]


@pytest.mark.parametrize("flags", [0, 1])
def test_ensemble_matches_single_runs(gpu_lib, flags):
    import hc
    cases = members()
    if flags:
        cases = [c for c in cases if c.params.imax == c.params.jmax]
    alone = []
    for c in cases:
        m = hc.Model(c)
        m.run(700, flags, records=False)
        alone.append(m)
    ens = [hc.Model(c) for c in cases]
    done = hc.run_ensemble(ens, 400, flags)
    done2 = hc.run_ensemble(ens, 300, flags)
    for k, (a, e) in enumerate(zip(alone, ens)):
        assert done[k] + done2[k] == 700, (k, done, done2)
        names = CHECK if not cases[k].params.hydro_only else CHECK[:6]
        for f in names:
            x, y = a.field(f), e.field(f)
            assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), (k, f)
        sa, se = a.scalars(), e.scalars()
        for s in ("cycle", "time_step", "maxdepth", "waterOut", "sediQ"):
            assert getattr(sa, s) == getattr(se, s), (k, s)
