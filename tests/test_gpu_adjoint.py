"""The adjoint of the hydraulic iteration (hc_adj_gradient) against central
finite differences of the same runs (hc_adj_forward with the time steps
imposed): directional derivatives of the outlet-discharge loss along random
seeded directions in Manning's n (32 of them, per cell), in the DEM and in
the rain table, to 1e-6 relative; forward-mode dual numbers; binomial
checkpointing against keeping every state; the torch.autograd.Function
wrapper (hc_torch.py)."""
import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu

WARM, N, EVERY = 250, 160, 48
REL = 1e-4     # central differences: the wider relative step
TOL = 1e-6     # adjoint against finite differences, relative


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
    loss, gn, gr, info = m.adj_gradient(N, EVERY, target)
    assert info["advanced"] == 0
    return case, target, rec, q, loss, gn, gr


def test_loss_matches_forward(setup):
    case, target, rec, q, loss, gn, gr = setup
    k = min(len(q), len(target))
    assert k > 5
    assert loss == pytest.approx(float(np.mean((q[:k] - target[:k]) ** 2)), rel=1e-12)
    assert np.abs(gn).max() > 0


def fd_pair(f, h, log=None):
    """Central differences at steps h and h/2, extrapolated (Richardson:
    the h^2 terms cancel): (estimate, consistent).  The two agree to the h^2
    term on a smooth stretch; a limiter or threshold that switches within
    the wider step (the depth limit and the hflow gate jump) makes them
    disagree far more, and the direction is skipped."""
    d1 = (f(h) - f(-h)) / (2 * h)
    d2 = (f(h / 2) - f(-h / 2)) / h
    if log is not None:
        log.append((d1, d2))
    return (4 * d2 - d1) / 3, abs(d1 - d2) <= 1e-5 * abs(d2) + 1e-15


def check_directions(ad_of, f_of, seeds, need):
    """Every direction whose finite differences are consistent must agree
    with the adjoint to 1e-6 relative; reports the skipped ones."""
    used, skipped, worst = 0, [], 0.0
    for seed in seeds:
        log = []
        fd, ok = fd_pair(f_of(seed), REL, log)
        if not ok:
            skipped.append(seed)
            print("direction %d skipped: differences %.6e (h) %.6e (h/2), adjoint %.6e"
                  % (seed, log[0][0], log[0][1], ad_of(seed)))
            continue
        ad = ad_of(seed)
        err = abs(ad - fd) / max(abs(fd), 1e-300)
        worst = max(worst, err)
        assert err <= TOL, (seed, ad, fd, err)
        used += 1
    print("directions used %d, skipped (a switch within the step) %s, worst rel %.2e"
          % (used, skipped, worst))
    assert used >= need, (used, skipped)


def test_manning_gradient_32_directions(setup):
    """32 seeded directions in Manning's n (relative perturbations of every
    cell) against central finite differences of the loss with the run's
    time steps imposed."""
    case, target, rec, q, loss, gn, gr = setup
    man = case.mannings

    def direction(seed):
        return np.random.default_rng(100 + seed).standard_normal(man.shape)

    def f_of(seed):
        v = direction(seed)
        return lambda h: loss_of(case, man * (1 + h * v), rec, target)

    def ad_of(seed):
        return float(np.sum(gn[1:-1, 1:-1] * man * direction(seed)))
    check_directions(ad_of, f_of, range(32), need=24)


def test_elevation_gradient_directions(setup_elev):
    """Directions in the DEM against central finite differences: 1e-3 m per
    unit of the direction, times REL (far below the jitter between
    neighbours, so that no pair of beds changes order)."""
    case, target, rec, loss, ge = setup_elev
    z = case.elev

    def direction(seed):
        return np.random.default_rng(200 + seed).standard_normal(z.shape) * 1e-3

    def f_of(seed):
        v = direction(seed)
        # a quarter of the n directions' step: at REL the input points
        # already change (an area crosses MIN_Q) in most directions
        return lambda h: elev_loss(case, z + (h / 4) * v, rec, target)

    def ad_of(seed):
        return float(np.sum(ge[1:-1, 1:-1] * direction(seed))) / 4
    check_directions(ad_of, f_of, range(12), need=4)


def elev_loss(case, elev_window, rec, target):
    m = warm_model(case)
    full = m.field("elev")
    full[1:-1, 1:-1] = elev_window
    m.upload("elev", full)
    _, q = m.adj_forward(N, fixed=rec)
    k = min(len(q), len(target))
    return float(np.mean((q[:k] - target[:k]) ** 2))


@pytest.fixture(scope="module")
def setup_elev(gpu_lib, setup):
    """The DEM with a seeded jitter below 1 mm: the pit filling leaves flats
    of exactly equal elevations, where max(e0, e1) has a kink that any
    perturbation of one of the two cells crosses (a central difference
    there averages the two one-sided derivatives)."""
    case0, target, rec0, q, loss0, gn, gr = setup
    case = base_case()
    rng = np.random.default_rng(23)
    case.elev = np.ascontiguousarray(case.elev + rng.uniform(0.0, 1e-3, case.elev.shape))
    rec, _ = warm_model(case).adj_forward(N)
    loss, gn2, gr2, info, ge = warm_model(case).adj_gradient(N, EVERY, target, elev=True)
    assert np.abs(ge).max() > 0
    return case, target, rec, loss, ge


def test_binomial_checkpointing_same_gradient(setup):
    """Few states kept (recomputation from snapshots) gives the gradient of
    the roomy run: Manning and elevation gradients bit for bit (the replayed
    iterations are the forward's own), the rain gradient to rounding (its
    per-zone sums are atomic)."""
    case, target, rec, q, loss, gn, gr = setup
    roomy = warm_model(case).adj_gradient(N, 400, target, elev=True)
    tight = warm_model(case).adj_gradient(N, 6, target, elev=True)
    assert tight[3]["advanced"] > 0 and roomy[3]["advanced"] == 0, (tight[3], roomy[3])
    assert tight[0] == roomy[0]
    np.testing.assert_array_equal(tight[1], roomy[1])
    np.testing.assert_array_equal(tight[4], roomy[4])
    np.testing.assert_allclose(tight[2], roomy[2], rtol=1e-12, atol=1e-300)


def test_autograd_function(setup):
    """hc_torch.OutletLoss: torch's backward gives the adjoint's gradients;
    the directional derivative along random directions in all three
    parameters matches central finite differences of problem.loss."""
    import torch
    import hc_torch
    case, target, rec, q, loss, gn, gr = setup
    prob = hc_torch.OutletLossProblem(case, WARM, N, target, max_states=EVERY)
    man = torch.tensor(case.mannings, dtype=torch.float64, requires_grad=True)
    elev = torch.tensor(case.elev, dtype=torch.float64, requires_grad=True)
    rain = torch.tensor(case.rain.astype(np.float64), dtype=torch.float64, requires_grad=True)
    out = hc_torch.OutletLoss.apply(man, elev, rain, prob)
    assert out.item() == pytest.approx(loss, rel=1e-12)
    out.backward()
    np.testing.assert_allclose(man.grad.numpy(), gn[1:-1, 1:-1], rtol=1e-12, atol=0)
    rng = np.random.default_rng(42)
    vn = rng.standard_normal(case.mannings.shape) * case.mannings
    ad = float((man.grad * torch.from_numpy(vn)).sum())
    fd, ok = fd_pair(lambda h: prob.loss(manning=case.mannings + h * vn, elev=case.elev), REL)
    assert ok
    assert ad == pytest.approx(fd, rel=TOL)


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
    lib.hco_dual_run.argtypes = ([C.c_int, C.c_int, d] + [vp] * 10 + [d, d, d, C.c_int, vp, i64,
                                 vp, C.c_int, vp, vp, d, d, C.c_int, d, d, d, d, d, vp, i64, vp,
                                 vp])
    return lib


def dual_check(case, rec, target, m, dman=None, delev=None):
    """(loss, directional derivative) of forward-mode dual numbers through a
    plain CPU restatement of the same iterations (oracle/hc_dual.cpp), from
    the warm model m's state, seeded with dman and/or delev."""
    import ctypes as C
    p = case.params
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
    rr = np.ascontiguousarray(rec)
    ts = np.ascontiguousarray(rec[:, 0])
    cyc = np.ascontiguousarray(rec[:, 21])
    tgt = np.ascontiguousarray(target)
    lo, dlo = C.c_double(), C.c_double()
    ptr = lambda a: None if a is None else a.ctypes.data
    return f, (lo, dlo), (p.imax, p.jmax, p.DX, ptr(f["elev"]), ptr(f["spat_var_mannings"]),
                          ptr(dman), ptr(delev), ptr(f["rfarea"]), ptr(f["water_depth"]),
                          ptr(f["qx"]), ptr(f["qy"]), ptr(mask), ptr(f["area"]), s.baseflow,
                          p.MIN_Q, p.MIN_Q_MAXVAL, p.rfnum, ptr(nact), N, ptr(rr), rr.shape[1],
                          ptr(ts), ptr(cyc), s.cycle, s.counter, p.scan_area_interval_iter,
                          p.hflow_threshold, p.froude_limit, p.edgeslope, p.ERODEFACTOR,
                          p.water_depth_erosion_threshold, ptr(tgt), len(tgt), C.byref(lo),
                          C.byref(dlo)), (rr, ts, cyc, tgt, mask, nact)


def test_manning_gradient_matches_dual_numbers(setup, dual_lib):
    """Forward-mode dual numbers through a plain CPU restatement of the same
    iterations (oracle/hc_dual.cpp), seeded with a direction in n."""
    case, target, rec, q, loss, gn, gr = setup
    m = warm_model(case)
    man = m.field("spat_var_mannings")
    rng = np.random.default_rng(5)
    v = np.zeros_like(man)
    v[1:-1, 1:-1] = rng.standard_normal((case.params.imax, case.params.jmax))
    dman = np.ascontiguousarray(man * v)
    f, (lo, dlo), args, keep = dual_check(case, rec, target, m, dman=dman)
    dual_lib.hco_dual_run(*args)
    assert lo.value == pytest.approx(loss, rel=1e-8)
    ad = float(np.sum(gn * dman))
    assert ad == pytest.approx(dlo.value, rel=1e-6)


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_elevation_gradient_matches_dual_numbers(setup_elev, dual_lib, seed):
    """The DEM gradient against dual numbers seeded with a direction in the
    elevations: exact derivatives along the run's own branches (which a
    central difference cannot isolate where a bed or surface maximum or a
    limiter sits on its switch)."""
    case, target, rec, loss, ge = setup_elev
    m = warm_model(case)
    v = np.zeros_like(ge)
    v[1:-1, 1:-1] = np.random.default_rng(300 + seed).standard_normal(
        (case.params.imax, case.params.jmax))
    delev = np.ascontiguousarray(v)
    f, (lo, dlo), args, keep = dual_check(case, rec, target, m, delev=delev)
    dual_lib.hco_dual_run(*args)
    assert lo.value == pytest.approx(loss, rel=1e-8)
    ad = float(np.sum(ge * delev))
    assert abs(dlo.value) > 0
    assert ad == pytest.approx(dlo.value, rel=1e-6)
