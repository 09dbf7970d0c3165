"""Seeded synthetic inputs for the benchmark and test workloads.

The reference ships only its Boscastle/Caersws fixtures; these generators make
DEMs, rain tables, reach hydrographs and Manning's n fields with the shapes,
sizes and value distributions of the benchmark configurations:

  reach_case      plain FP64 reach-mode run: inclined V-valley with a
                  rectangular channel, one upstream inflow point carrying a
                  triangular hydrograph, Wilcock-Crowe transport
  catchment_case  catchment mode: spectral-fractal DEM, pit-filled toward
                  one outlet edge, gamma-distributed rain plus a storm,
                  per-cell Manning's n, Einstein transport
  flow_case       flow-only bandwidth case: fractal DEM, uniform rain

Everything is deterministic in its seed.  Arrays are unpadded (imax, jmax);
the model pads them (LSDCatchmentModel.cpp:190-196).
"""
import heapq
import numpy as np

from hc_abi import default_params


class Case:
    """One model set-up: parameters, rasters and time series."""

    def __init__(self, name, params, elev, rain, reach=None, mannings=None,
                 water_init=None, flags=0):
        self.name = name
        self.params = params
        self.elev = np.ascontiguousarray(elev, dtype=np.float64)
        self.rain = np.ascontiguousarray(rain, dtype=np.float32)
        self.reach = [np.ascontiguousarray(r, dtype=np.float32) for r in (reach or [])]
        self.mannings = None if mannings is None else np.ascontiguousarray(mannings, np.float64)
        self.water_init = None if water_init is None else np.ascontiguousarray(water_init, np.float64)
        self.flags = flags

    @property
    def cells(self):
        return self.params.imax * self.params.jmax


# ---------------------------------------------------------------- fields
def correlated_noise(shape, sigma, corr_len_cells, rng):
    """Gaussian white noise low-passed by a Gaussian kernel in Fourier space,
    rescaled to standard deviation sigma."""
    w = rng.standard_normal(shape)
    ky = np.fft.fftfreq(shape[0])[:, None]
    kx = np.fft.rfftfreq(shape[1])[None, :]
    filt = np.exp(-2.0 * (np.pi * corr_len_cells) ** 2 * (kx ** 2 + ky ** 2))
    f = np.fft.irfft2(np.fft.rfft2(w) * filt, s=shape)
    f -= f.mean()
    s = f.std()
    return f * (sigma / s) if s > 0 else f


def fractal_surface(shape, beta, rng):
    """Spectral synthesis: power spectrum ~ k^-beta, zero mean, unit range."""
    ky = np.fft.fftfreq(shape[0])[:, None]
    kx = np.fft.rfftfreq(shape[1])[None, :]
    k = np.sqrt(kx ** 2 + ky ** 2)
    k[0, 0] = 1.0
    amp = k ** (-beta / 2.0)
    amp[0, 0] = 0.0
    phase = rng.uniform(0, 2 * np.pi, amp.shape)
    mag = rng.standard_normal(amp.shape)
    spec = amp * mag * np.exp(1j * phase)
    f = np.fft.irfft2(spec, s=shape)
    f -= f.min()
    rng_ = f.max()
    return f / rng_ if rng_ > 0 else f


def fill_pits(z, outlet_edge="bottom", eps=1e-4):
    """Priority-flood (Barnes et al. 2014, with an epsilon gradient) seeded
    from one edge, so every cell drains to that edge."""
    imax, jmax = z.shape
    out = z.copy()
    done = np.zeros(z.shape, dtype=bool)
    heap = []
    if outlet_edge == "bottom":
        seeds = [(imax - 1, j) for j in range(jmax)]
    elif outlet_edge == "top":
        seeds = [(0, j) for j in range(jmax)]
    elif outlet_edge == "left":
        seeds = [(i, 0) for i in range(imax)]
    else:
        seeds = [(i, jmax - 1) for i in range(imax)]
    for (i, j) in seeds:
        heapq.heappush(heap, (out[i, j], i, j))
        done[i, j] = True
    nb = [(-1, -1), (-1, 0), (-1, 1), (0, -1), (0, 1), (1, -1), (1, 0), (1, 1)]
    while heap:
        h, i, j = heapq.heappop(heap)
        for di, dj in nb:
            a, b = i + di, j + dj
            if 0 <= a < imax and 0 <= b < jmax and not done[a, b]:
                done[a, b] = True
                if out[a, b] <= h:
                    out[a, b] = h + eps
                heapq.heappush(heap, (out[a, b], a, b))
    return out


def fractal_dem(imax, jmax, relief, seed, beta=2.0, outlet_edge="bottom", tilt=0.25,
                fill=True):
    """Fractal DEM scaled to `relief` m, tilted toward the outlet edge by
    `tilt` x relief, optionally pit-filled toward it."""
    rng = np.random.default_rng(seed)
    f = fractal_surface((imax, jmax), beta, rng)
    ramp = np.linspace(1.0, 0.0, imax)[:, None] * np.ones((1, jmax))
    if outlet_edge == "top":
        ramp = ramp[::-1]
    z = (1.0 - tilt) * f + tilt * ramp
    z -= z.min()
    z *= relief / z.max()
    z += 10.0
    if fill:
        z = fill_pits(z, outlet_edge)
    return np.round(z, 6)


def lognormal_dprop(d, median, sigma_ln=1.0):
    """Grain-size proportions: log-normal weights at the 9 sizes d[1..9],
    normalised to sum 1 (dprop[0] = dprop[10] = 0)."""
    x = np.log(np.asarray(d[1:10]) / median)
    w = np.exp(-0.5 * (x / sigma_ln) ** 2)
    w /= w.sum()
    out = [0.0] + list(w) + [0.0]
    return out


def geometric_sizes(lo=0.001, hi=0.256):
    r = (hi / lo) ** (1.0 / 8.0)
    return [0.0] + [lo * r ** k for k in range(9)]


def set_grains(p, sizes, dprop):
    for n in range(10):
        p.d[n] = sizes[n]
    for n in range(11):
        p.dprop[n] = dprop[n]


# ---------------------------------------------------------------- time series
def zero_rain_table(p):
    """hourly_rain_data when no rain file is read (LSDCatchmentModel.cpp:1699)."""
    rows = int(p.maxcycle * (60 / p.rain_data_time_step)) + 100
    return np.zeros((rows, p.rfnum + 1), dtype=np.float32)


def triangular_hydrograph(q0, qpeak, t_peak_h, t_end_h, dt_min, rows):
    t = np.arange(rows) * dt_min / 60.0
    q = np.where(t <= t_peak_h, q0 + (qpeak - q0) * t / t_peak_h,
                 qpeak - (qpeak - q0) * (t - t_peak_h) / (t_end_h - t_peak_h))
    q = np.where(t > t_end_h, q0, q)
    return q


# ---------------------------------------------------------------- cases
def reach_case(imax=300, jmax=100, DX=10.0, seed=1, hours=24, hydro_only=False):
    """Reach mode: rows are the downstream direction.  Plane sloping 0.005
    along the rows, V cross-section (side slope 0.05), a 20 m x 2 m channel
    on the centreline, correlated noise (sigma 0.05 m, 50 m); one inflow
    cell near the upstream end with a 5->150->5 m3/s hydrograph peaking at
    6 h over 24 h (1-min table)."""
    rng = np.random.default_rng(seed)
    i = np.arange(imax)[:, None]
    j = np.arange(jmax)[None, :]
    jc = (jmax - 1) / 2.0
    z = 50.0 - 0.005 * DX * i + 0.05 * DX * np.abs(j - jc)
    chan_half = max(1, int(round(10.0 / DX)))
    chan = np.abs(j - jc) <= chan_half - 0.5 + 1e-9
    z = z - 2.0 * chan
    z = z + correlated_noise((imax, jmax), 0.05, 50.0 / DX, rng)
    z = np.round(z, 6)
    p = default_params(imax, jmax, DX)
    p.maxcycle = hours
    p.max_time_step = 300
    p.courant_number = 0.7
    p.mannings = 0.04
    p.hydro_only = 1 if hydro_only else 0
    p.wilcock, p.einstein = 1, 0
    p.active = 0.2
    p.edgeslope = 0.005
    p.M = 0.005
    p.MIN_Q = 0.01
    p.reach_mode = 1
    p.number_of_points = 1
    p.inpoints[0][0] = 3
    p.inpoints[0][1] = int(round(jc)) + 1
    p.reach_input_data_timestep = 1
    p.rain_data_time_step = 60
    sizes = geometric_sizes(0.001, 0.256)
    set_grains(p, sizes, lognormal_dprop(sizes, 0.016))
    rows = hours * 60 + 200
    q = triangular_hydrograph(5.0, 150.0, 6.0, 24.0, 1.0, rows)
    table = np.zeros((rows, 16), dtype=np.float32)
    table[:, 0] = np.arange(rows)
    table[:, 1] = q
    rain = zero_rain_table(p)
    return Case("reach_%dx%d" % (imax, jmax), p, z, rain, reach=[table])


def gamma_rain(hours, step_min, mean_mmh, shape_k, storm_mmh, storm_start_h,
               storm_len_h, seed, pad_rows=200):
    rng = np.random.default_rng(seed)
    rows = int(hours * 60 / step_min) + pad_rows
    r = rng.gamma(shape_k, mean_mmh / shape_k, rows)
    s0 = int(storm_start_h * 60 / step_min)
    s1 = int((storm_start_h + storm_len_h) * 60 / step_min)
    r[s0:s1] = storm_mmh
    return r.astype(np.float32)[:, None]


def catchment_case(n=2000, DX=20.0, seed=2, hours=72, lateral=True, hydro_only=False,
                   jmax=None, relief=300.0, fill=True, storm_start_h=12.0):
    """Catchment mode: fractal DEM (beta 2, `relief` m) pit-filled toward the
    bottom edge; rain in 10-min steps ~ gamma(k=0.5, mean 2 mm/h) plus a
    60 mm/h storm of 3 h starting at `storm_start_h`; TOPMODEL m = 0.01; Manning's n from a smooth field
    in [0.03, 0.06]; Einstein transport; slide_3 (always on with erosion) and
    lateral3 (called after erosion)."""
    imax = n
    jmax = n if jmax is None else jmax
    z = fractal_dem(imax, jmax, relief, seed, fill=fill)
    rng = np.random.default_rng(seed + 1000)
    nf = correlated_noise((imax, jmax), 1.0, max(2.0, imax / 20.0), rng)
    nf = (nf - nf.min()) / max(1e-12, nf.max() - nf.min())
    man = np.round(0.03 + 0.03 * nf, 6)
    p = default_params(imax, jmax, DX)
    p.maxcycle = hours
    p.max_time_step = 300
    p.rain_data_time_step = 10
    p.M = 0.01
    p.spatially_var_mannings = 1
    p.hydro_only = 1 if hydro_only else 0
    p.wilcock, p.einstein = 0, 1
    p.active = 0.2
    p.edgeslope = 0.005
    p.MIN_Q = 0.01
    sizes = geometric_sizes(0.001, 0.256)
    set_grains(p, sizes, lognormal_dprop(sizes, 0.016))
    rain = gamma_rain(hours, 10, 2.0, 0.5, 60.0, storm_start_h, 3.0, seed + 2000)
    flags = 1 if lateral else 0
    return Case("catchment_%dx%d" % (imax, jmax), p, z, rain, mannings=man, flags=flags)


def flow_case(n=8192, DX=5.0, seed=3, hours=2, rain_mmh=30.0, jmax=None, relief=150.0,
              fill=False, grid_rain=False):
    """Flow-only bandwidth case: fractal DEM at `relief` m, uniform rain
    `rain_mmh` for `hours` h, erosion off.  grid_rain: the rain reaches every
    cell (the distributed TOPMODEL runoff grid, spatially_complex_rainfall)
    instead of the drainage network's input points, so the whole grid is
    wet."""
    imax = n
    jmax = n if jmax is None else jmax
    z = fractal_dem(imax, jmax, relief, seed, fill=fill)
    p = default_params(imax, jmax, DX)
    p.maxcycle = hours + 1
    p.max_time_step = 300
    p.rain_data_time_step = 60
    p.hydro_only = 1
    p.M = 0.005
    p.edgeslope = 0.005
    if grid_rain:
        p.spatially_complex_rainfall = 1
    rows = int(p.maxcycle * 60 / p.rain_data_time_step) + 100
    rain = np.zeros((rows, 1), dtype=np.float32)
    rain[: hours] = rain_mmh
    return Case("flow_%dx%d" % (imax, jmax), p, z, rain)


def adjoint_case(n=1024, DX=10.0, seed=4, relief=200.0, rain_mmh=20.0, storm_h=3, hours=12,
                 fill=True, n_seed=None):
    """Hydro-only catchment for the adjoint: fractal DEM (`relief` m),
    uniform rain `rain_mmh` for the first `storm_h` hours in 10-min steps,
    Manning's n from a smooth seeded field in [0.03, 0.06] (n_seed: another
    field, for a target run)."""
    z = fractal_dem(n, n, relief, seed, fill=fill)
    rng = np.random.default_rng((seed if n_seed is None else n_seed) + 1000)
    nf = correlated_noise((n, n), 1.0, max(2.0, n / 20.0), rng)
    nf = (nf - nf.min()) / max(1e-12, nf.max() - nf.min())
    man = np.round(0.03 + 0.03 * nf, 6)
    p = default_params(n, n, DX)
    p.maxcycle = hours
    p.max_time_step = 300
    p.rain_data_time_step = 10
    p.M = 0.01
    p.spatially_var_mannings = 1
    p.hydro_only = 1
    p.edgeslope = 0.005
    p.MIN_Q = 0.01
    rows = int(hours * 60 / 10) + 200
    rain = np.zeros((rows, 1), dtype=np.float32)
    rain[: storm_h * 6] = rain_mmh
    return Case("adjoint_%dx%d" % (n, n), p, z, rain, mannings=man, flags=0)


def ensemble_member(k, seed=5, DX=10.0, hours=12, side_min=256, side_max=1536, fill=True):
    """Member k of the ensemble: sides U[side_min, side_max] per axis,
    relief U[100, 400] m, uniform rain U[5, 50] mm/h for the first 4 h, one
    Manning's n U[0.02, 0.08]; flow and erosion (Einstein, 9 fractions,
    slide_3), no lateral3 (members need not be square)."""
    rng = np.random.default_rng(seed * 100003 + k)
    imax = int(rng.integers(side_min, side_max + 1))
    jmax = int(rng.integers(side_min, side_max + 1))
    relief = float(rng.uniform(100.0, 400.0))
    rain_mmh = float(rng.uniform(5.0, 50.0))
    n_man = float(np.round(rng.uniform(0.02, 0.08), 6))
    z = fractal_dem(imax, jmax, relief, seed * 7919 + k, fill=fill)
    p = default_params(imax, jmax, DX)
    p.maxcycle = hours
    p.max_time_step = 300
    p.rain_data_time_step = 10
    p.M = 0.01
    p.mannings = n_man
    p.wilcock, p.einstein = 0, 1
    p.active = 0.2
    p.edgeslope = 0.005
    p.MIN_Q = 0.01
    sizes = geometric_sizes(0.001, 0.256)
    set_grains(p, sizes, lognormal_dprop(sizes, 0.016))
    rows = int(hours * 60 / 10) + 200
    rain = np.zeros((rows, 1), dtype=np.float32)
    rain[: 4 * 6] = rain_mmh
    return Case("member%d_%dx%d" % (k, imax, jmax), p, z, rain, flags=0)


# ---------------------------------------------------------------- padding
def padded(case, a, fill):
    p = case.params
    out = np.full((p.imax + 2, p.jmax + 2), fill, dtype=np.float64)
    out[1:-1, 1:-1] = a
    return out
