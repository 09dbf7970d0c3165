"""Comparison helpers shared by the parity tests."""
import numpy as np

HYDRO_FIELDS = ["elev", "water_depth", "qx", "qy", "qxs", "qys", "Vsusptot", "down_scan",
                "vel_dir"]
SED_FIELDS = ["Vel", "Tau", "ss", "index", "grain", "strata", "sr", "sl", "su", "sd", "edge"]


def state_of(model_or_oracle, names):
    return {k: np.array(model_or_oracle.field(k), copy=True) for k in names}


def max_abs_diff(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.abs(a - b)
    d[both_nan] = 0
    return float(np.nanmax(d)) if d.size else 0.0


def assert_bitwise(got, want, name):
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape, (name, got.shape, want.shape)
    if got.dtype.kind == "f":
        same = (got == want) | (np.isnan(got) & np.isnan(want))
    else:
        same = got == want
    if not same.all():
        idx = np.argwhere(~same)
        first = tuple(idx[0])
        raise AssertionError("%s: %d mismatches, first at %s: got %r want %r (max abs diff %.3e)"
                             % (name, len(idx), first, got[first], want[first],
                                max_abs_diff(got, want)))


def assert_close(got, want, atol, name, rtol=0.0):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape, (name, got.shape, want.shape)
    ok = np.isclose(got, want, atol=atol, rtol=rtol, equal_nan=True)
    if not ok.all():
        idx = np.argwhere(~ok)
        first = tuple(idx[0])
        raise AssertionError("%s: %d cells beyond atol %.1e rtol %.1e, first at %s: got %r want %r"
                             % (name, len(idx), atol, rtol, first, got[first], want[first]))
