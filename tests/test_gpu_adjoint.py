"""The adjoint of the hydraulic iteration (hc_adj_gradient) against central
finite differences of the same runs (hc_adj_forward with the time steps
imposed): directional derivatives of the outlet-discharge loss along random
seeded directions in Manning's n (per cell) and in the rain table."""
import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu

WARM, N, EVERY = 250, 160, 48
REL = 1e-6     # central differences, relative step


def base_case(rain=None, man=None):
    case = synth.catchment_case(n=40, DX=20.0, hours=72, relief=60.0, hydro_only=True,
                                lateral=False, storm_start_h=0.2)
    if rain is not None:
        case.rain = np.ascontiguousarray(rain, dtype=np.float32)
    if man is not None:
        case.mannings = np.ascontiguousarray(man)
    return case


def warm_model(case):
    import hc
    m = hc.Model(case)
    m.run(WARM, records=False)
    return m


def loss_of(case, man_window, rec, target):
    m = warm_model(case)
    p = case.params
    full = np.zeros((p.imax + 2, p.jmax + 2))
    full[1:-1, 1:-1] = man_window
    m.upload("spat_var_mannings", full)
    _, q = m.adj_forward(N, fixed=rec)
    k = min(len(q), len(target))
    return float(np.mean((q[:k] - target[:k]) ** 2))


@pytest.fixture(scope="module")
def setup(gpu_lib):
    case = base_case()
    # target: the same catchment with another Manning field
    rng = np.random.default_rng(11)
    tcase = base_case(man=case.mannings * (1.0 + 0.3 * rng.random(case.mannings.shape)))
    _, target = warm_model(tcase).adj_forward(N)
    rec, q = warm_model(case).adj_forward(N)
    m = warm_model(case)
    loss, gn, gr, ms = m.adj_gradient(N, EVERY, target)
    return case, target, rec, q, loss, gn, gr


def test_loss_matches_forward(setup):
    case, target, rec, q, loss, gn, gr = setup
    k = min(len(q), len(target))
    assert k > 5
    assert loss == pytest.approx(float(np.mean((q[:k] - target[:k]) ** 2)), rel=1e-12)
    assert np.abs(gn).max() > 0


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_manning_gradient_matches_finite_differences(setup, seed):
    case, target, rec, q, loss, gn, gr = setup
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(case.mannings.shape)
    man = case.mannings
    h = REL
    lp = loss_of(case, man * (1 + h * v), rec, target)
    lm = loss_of(case, man * (1 - h * v), rec, target)
    fd = (lp - lm) / (2 * h)
    ad = float(np.sum(gn[1:-1, 1:-1] * man * v))
    assert ad == pytest.approx(fd, rel=2e-4, abs=1e-9 * max(1.0, abs(loss)))


def test_rain_gradient_matches_finite_differences(setup):
    case, target, rec, q, loss, gn, gr = setup
    rain = case.rain.astype(np.float64)
    # rows after the warm-up (earlier rows also moved the warm-up state)
    first = int(np.ceil(rec[0, 20] / case.params.rain_data_time_step)) + 1
    rng = np.random.default_rng(7)
    v = np.zeros_like(rain)
    rows = slice(first, first + 12)
    v[rows] = rng.standard_normal(v[rows].shape) * (rain[rows] > 0)
    h = 1e-4
    rp = (rain * (1 + h * v)).astype(np.float32)
    rm = (rain * (1 - h * v)).astype(np.float32)

    def loss_rain(r):
        c = base_case(rain=r)
        return loss_of(c, c.mannings, rec, target)
    fd = (loss_rain(rp) - loss_rain(rm)) / 2
    ad = float(np.sum(gr * (rp.astype(np.float64) - rm.astype(np.float64)))) / 2
    assert ad == pytest.approx(fd, rel=2e-3, abs=1e-12 * max(1.0, abs(loss)))


# ---------------------------------------------------------------- dual numbers
@pytest.fixture(scope="module")
def dual_lib(tmp_path_factory):
    import ctypes as C
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    so = str(tmp_path_factory.mktemp("dual") / "hc_dual.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", so,
                    os.path.join(root, "oracle", "hc_dual.cpp")], check=True)
    lib = C.CDLL(so)
    vp, i64, d = C.c_void_p, C.c_int64, C.c_double
    lib.hco_dual_run.restype = C.c_int
    lib.hco_dual_run.argtypes = ([C.c_int, C.c_int, d] + [vp] * 9 + [d, d, d, C.c_int, vp, i64,
                                 vp, C.c_int, vp, vp, d, d, C.c_int, d, d, d, d, d, vp, i64, vp,
                                 vp])
    return lib


def test_manning_gradient_matches_dual_numbers(setup, dual_lib):
    """Forward-mode dual numbers through a plain CPU restatement of the same
    iterations (oracle/hc_dual.cpp), seeded with a direction in n."""
    import ctypes as C
    case, target, rec, q, loss, gn, gr = setup
    p = case.params
    m = warm_model(case)
    s = m.scalars()
    f = {k: np.ascontiguousarray(m.field(k)) for k in
         ("water_depth", "qx", "qy", "elev", "spat_var_mannings", "rfarea", "area")}
    ds = m.field("down_scan")
    mask = np.zeros((p.imax + 2, p.jmax + 2), dtype=np.uint8)
    for j in range(1, p.jmax + 1):
        for k in range(1, p.imax + 2):
            i = ds[j, k]
            if i <= 0:
                break
            mask[i, j] = 1
    nact = np.array(list(s.nActualGridCells), dtype=np.float64)
    rng = np.random.default_rng(5)
    v = np.zeros_like(f["spat_var_mannings"])
    v[1:-1, 1:-1] = rng.standard_normal((p.imax, p.jmax))
    dman = np.ascontiguousarray(f["spat_var_mannings"] * v)
    rr = np.ascontiguousarray(rec)
    ts = np.ascontiguousarray(rec[:, 0])
    cyc = np.ascontiguousarray(rec[:, 21])
    tgt = np.ascontiguousarray(target)
    lo, dlo = C.c_double(), C.c_double()
    ptr = lambda a: a.ctypes.data
    dual_lib.hco_dual_run(p.imax, p.jmax, p.DX, ptr(f["elev"]), ptr(f["spat_var_mannings"]),
                          ptr(dman), ptr(f["rfarea"]), ptr(f["water_depth"]), ptr(f["qx"]),
                          ptr(f["qy"]), ptr(mask), ptr(f["area"]), s.baseflow, p.MIN_Q,
                          p.MIN_Q_MAXVAL, p.rfnum, ptr(nact), N, ptr(rr), rr.shape[1], ptr(ts),
                          ptr(cyc), s.cycle, s.counter,
                          p.scan_area_interval_iter, p.hflow_threshold, p.froude_limit,
                          p.edgeslope, p.ERODEFACTOR, p.water_depth_erosion_threshold, ptr(tgt),
                          len(tgt), C.byref(lo), C.byref(dlo))
    assert lo.value == pytest.approx(loss, rel=1e-8)
    ad = float(np.sum(gn * dman))
    assert ad == pytest.approx(dlo.value, rel=1e-6)
