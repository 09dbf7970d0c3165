"""The drainage sweep order sorted on the device (hc_sort.cu) against the
permutation std::sort gives the same pairs (the oracle calls the library
sort the reference calls, LSDCatchmentModel.cpp:2143-2180), equal values
included; and the drainage area of a model whose flats make that order
matter."""
import numpy as np
import pytest

import synth
from helpers import assert_bitwise

pytestmark = pytest.mark.gpu


def std_perm(oracle_mod, v):
    lib = oracle_mod._lib()
    v = np.ascontiguousarray(v, dtype=np.float64)
    perm = np.empty(v.size, np.uint32)
    lib.hco_sort_perm(v.ctypes.data, v.size, perm.ctypes.data)
    return perm


def inputs():
    rng = np.random.default_rng(11)
    for n in (0, 1, 2, 15, 16, 17, 33, 100, 1000, 4096, 4097, 5000, 70000, 300000, 2_000_000):
        yield n, "few ties", rng.integers(0, 1_000_000, n) * 1e-3
        yield n, "heavy ties", rng.integers(0, 7, n).astype(float)
        yield n, "sorted", np.arange(n, dtype=float)
        yield n, "reversed", np.arange(n, 0, -1, dtype=float)
        yield n, "all equal", np.full(n, 5.0)
        yield n, "no-data and flats", np.where(np.arange(n) % 97 == 0, -9999.0,
                                               100 + rng.integers(0, 50, n) * 0.5)
        yield n, "signed zeros", rng.choice([-0.0, 0.0, 1.0, -1.0], n)


def padded(z):
    """drainage_area_D8's pair vector: (imax+2)(jmax+2) values, 0 except
    positions 1 .. imax*jmax, which hold the elevations row by row."""
    imax, jmax = z.shape
    v = np.zeros((imax + 2) * (jmax + 2))
    v[1:1 + imax * jmax] = z.ravel()
    return v


def test_sort_matches_std_sort(gpu_lib, oracle_mod):
    import hc
    bad = []
    for n, kind, v in inputs():
        perm, on_device = hc.drainage_sort(v)
        assert on_device, (n, kind)
        ref = std_perm(oracle_mod, v)
        if not np.array_equal(perm, ref):
            k = int(np.argmax(perm != ref))
            bad.append("%s n=%d first difference at %d" % (kind, n, k))
    assert not bad, bad


def test_sort_terrain_pair_vectors(gpu_lib, oracle_mod):
    """Pit-filled catchments (flats: long runs of equal elevations), with
    and without no-data margins, in the reference's padded layout."""
    import hc
    for n, step in ((300, 0.5), (1000, 0.25), (2000, 0.5)):
        case = synth.catchment_case(n=n, DX=20.0, hours=1, relief=60.0, hydro_only=True,
                                    lateral=False)
        z = np.round(case.elev / step) * step
        for margin in (0, 7):
            zz = z.copy()
            if margin:
                zz[:, :margin] = -9999.0
            v = padded(zz)
            perm, on_device = hc.drainage_sort(v)
            assert on_device, n
            assert_bitwise(perm, std_perm(oracle_mod, v), "order n=%d margin=%d" % (n, margin))


def test_sort_depth_budget_falls_back(gpu_lib, oracle_mod):
    """An organ-pipe input drives median-of-three quicksort into std::sort's
    heapsort branch; the device declines and the host's exact sort answers."""
    import hc
    n = 70000
    k = np.arange(n)
    v = np.where(k < n // 2, k, n - k).astype(float)
    perm, on_device = hc.drainage_sort(v)
    assert not on_device
    assert_bitwise(perm, std_perm(oracle_mod, v), "order")


def test_model_area_with_device_sort(gpu_lib, oracle_mod):
    """A 160 x 160 catchment on a 0.5 m grid of elevations: the sweep order
    (26,244 pairs, split grid-wide before the block phase) decides the order
    of equal-elevation pushes; areas match the reference bit for bit and the
    sort ran on the device."""
    import hc
    case = synth.catchment_case(n=160, DX=20.0, hours=72, relief=60.0, hydro_only=True,
                                lateral=False, storm_start_h=0.5)
    case.elev = np.ascontiguousarray(np.round(case.elev * 2) / 2)
    m = hc.Model(case)
    m.run(300)
    o = oracle_mod.Oracle(case)
    o.iterate(300)
    assert_bitwise(m.field("area"), o.field("area"), "area")
    st = m.run_stats()
    assert st["drainage_sort"][0] >= 1, st
    assert st["drainage_host_sort"][0] == 0, st
