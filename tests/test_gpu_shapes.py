"""k_flow_route's launch shapes (register budgets, grids, and the
face-compacted kernel) compute the same discharges bit for bit, and the
autotuner that picks one leaves the model state as it found it."""
import numpy as np
import pytest

import synth
from helpers import assert_bitwise

pytestmark = pytest.mark.gpu

SHAPES = 18
FIELDS = ("water_depth", "qx", "qy", "qxs", "qys", "Vsusptot", "elev", "vel_dir", "index")


def storm_case(hydro_only):
    return synth.catchment_case(n=96, DX=20.0, hours=72, relief=60.0, hydro_only=hydro_only,
                                lateral=False, storm_start_h=0.3)


@pytest.mark.parametrize("hydro_only", [False, True])
def test_every_shape_gives_the_same_run(gpu_lib, hydro_only):
    import hc
    case = storm_case(hydro_only)
    fields = FIELDS if not hydro_only else ("water_depth", "qx", "qy")
    ref = hc.Model(case)
    ref.set_launch_shape(0)
    ra = ref.run(600)
    want = {k: ref.field(k) for k in fields}
    for shape in range(1, SHAPES):
        m = hc.Model(case)
        m.set_launch_shape(shape)
        rb = m.run(600)
        assert_bitwise(rb, ra, "records, shape %d" % shape)
        for k in fields:
            assert_bitwise(m.field(k), want[k], "%s, shape %d" % (k, shape))
        m.close()


def test_tuning_leaves_the_state_alone(gpu_lib):
    import hc
    case = storm_case(False)
    a = hc.Model(case)
    ra = np.concatenate([a.run(300), a.run(300)])
    b = hc.Model(case)
    r1 = b.run(300)
    shape, ms = b.autotune(force=True)
    assert 0 <= shape < SHAPES and min(ms) > 0
    rb = np.concatenate([r1, b.run(300)])
    assert_bitwise(rb, ra, "records")
    for k in FIELDS:
        assert_bitwise(b.field(k), a.field(k), k)
