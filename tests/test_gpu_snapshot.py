"""hc_snapshot_begin / hc_snapshot_end: a field copied while the run goes
on equals the field at the moment the snapshot was taken."""
import numpy as np
import pytest
import torch

import synth

pytestmark = pytest.mark.gpu


def test_snapshot_is_the_field_when_taken(gpu_lib):
    import hc
    case = synth.catchment_case(n=48, DX=20.0, hours=72, relief=60.0, lateral=False,
                                storm_start_h=0.2)
    a, b = hc.Model(case), hc.Model(case)
    a.run(300, records=False)
    b.run(300, records=False)
    ref = {k: b.field(k) for k in ("water_depth", "elev", "qx")}
    outs = {k: torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy()
            for k, v in ref.items()}
    handles = [a.snapshot_begin(k, outs[k]) for k in ref]
    a.run(200, records=False)  # the run goes on meanwhile
    for h in handles:
        a.snapshot_end(h)
    for k in ref:
        assert np.array_equal(outs[k].view(np.uint8), ref[k].view(np.uint8)), k
    assert not np.array_equal(a.field("water_depth"), ref["water_depth"])
