"""Host-side mirror of the reference's hot-path members over libhc_gpu.

`Model` holds one device-resident model state and exposes the members that
src/main.cpp calls each iteration (flow_route, depth_update, scan_area,
erode, lateral_channel_erode, in_channel_landsliding, water_flux_out, ...)
plus `run`, which executes whole iterations of the main loop on the device.
It is a thin ctypes layer: every call goes through the C ABI of
include/hc_gpu.h, the same entry points a C++ caller binds.  There is no CPU
fallback: constructing a Model without the built library raises.
"""
import ctypes as C
import os

import numpy as np

from hc_abi import (hc_params, hc_scalars, hc_step_record, hc_mass, FIELD_ID, STATUS,
                    STEP_FIELDS, field_shape, field_dtype)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhc_gpu.so")

_lib = None


class HCError(RuntimeError):
    pass


def load_library(path=LIB_PATH):
    """Loads libhc_gpu.so (built by build.py) and declares its ABI."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise HCError("libhc_gpu.so is not built (run hail-caesar_gb300/build.py): " + path)
    lib = C.CDLL(path)
    P, vp = C.POINTER, C.c_void_p
    sig = {
        "hc_params_default": (None, [P(hc_params), C.c_int32, C.c_int32, C.c_double]),
        "hc_field_count": (C.c_int64, [P(hc_params), C.c_int]),
        "hc_field_elsize": (C.c_int32, [C.c_int]),
        "hc_create": (C.c_int, [P(hc_params), C.c_size_t, P(vp)]),
        "hc_destroy": (C.c_int, [vp]),
        "hc_last_error": (C.c_char_p, [vp]),
        "hc_upload": (C.c_int, [vp, C.c_int, vp, C.c_size_t]),
        "hc_download": (C.c_int, [vp, C.c_int, vp, C.c_size_t]),
        "hc_set_rain": (C.c_int, [vp, vp, C.c_int32, C.c_int32]),
        "hc_set_reach": (C.c_int, [vp, C.c_int32, vp, C.c_int32, C.c_int32]),
        "hc_get_scalars": (C.c_int, [vp, P(hc_scalars)]),
        "hc_set_scalars": (C.c_int, [vp, P(hc_scalars)]),
        "hc_prepare": (C.c_int, [vp]),
        "hc_set_maximum_timestep": (C.c_int, [vp]),
        "hc_flow_route": (C.c_int, [vp]),
        "hc_depth_update": (C.c_int, [vp]),
        "hc_scan_area": (C.c_int, [vp]),
        "hc_water_flux_out": (C.c_int, [vp]),
        "hc_erode": (C.c_int, [vp, C.c_double, P(C.c_double)]),
        "hc_lateral_channel_erode": (C.c_int, [vp]),
        "hc_in_channel_landsliding": (C.c_int, [vp]),
        "hc_global_landsliding": (C.c_int, [vp, P(C.c_int32)]),
        "hc_creep": (C.c_int, [vp, C.c_double]),
        "hc_run": (C.c_int, [vp, C.c_int64, C.c_int32, vp, P(C.c_int64)]),
        "hc_stream": (vp, [vp]),
        "hc_run_ensemble": (C.c_int, [P(vp), C.c_int32, C.c_int64, C.c_int32, P(C.c_int64)]),
        "hc_bench_kernel": (C.c_int, [vp, C.c_char_p, C.c_int32, P(C.c_double), P(C.c_int64)]),
        "hc_get_counters": (C.c_int, [vp, P(C.c_int64), P(C.c_int64), P(C.c_int64)]),
        "hc_get_run_stats": (C.c_int, [vp, P(C.c_int64), P(C.c_double), C.c_int32]),
        "hc_snapshot_begin": (C.c_int, [vp, C.c_int, vp, C.c_size_t, P(vp)]),
        "hc_snapshot_end": (C.c_int, [vp]),
        "hc_adj_forward": (C.c_int, [vp, C.c_int64, vp, vp, vp, C.c_int64, P(C.c_int64)]),
        "hc_adj_gradient": (C.c_int, [vp, C.c_int64, C.c_int32, vp, C.c_int64, P(C.c_double),
                                      vp, vp, vp, vp]),
        "hc_profile_iteration": (C.c_int, [vp, C.c_int32, P(C.c_double)]),
        "hc_drainage_sort": (C.c_int, [vp, C.c_uint64, vp, P(C.c_int32)]),
        "hc_mass_balance": (C.c_int, [vp, P(hc_mass)]),
        "hc_mass_reset": (C.c_int, [vp]),
        "hc_test_bounded_waits": (C.c_int, [vp, C.c_int32, C.c_int32]),
        "hc_autotune": (C.c_int, [vp, C.c_int32, P(C.c_int32), P(C.c_double), C.c_int32]),
        "hc_set_launch_shape": (C.c_int, [vp, C.c_int32]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def drainage_sort(values):
    """(perm, on_device): the permutation std::sort gives (index, value)
    pairs compared by value, as drainage_area_D8 sorts its elevations;
    on_device False when the host's exact sort ran instead."""
    lib = load_library()
    v = np.ascontiguousarray(values, dtype=np.float64)
    perm = np.empty(v.size, dtype=np.uint32)
    dev = C.c_int32(1)
    st = lib.hc_drainage_sort(v.ctypes.data, v.size, perm.ctypes.data, C.byref(dev))
    if st != 0:
        raise HCError("drainage_sort failed: %s" % STATUS.get(st, st))
    return perm, bool(dev.value)


class Model:
    """One model state on the GPU, set up from a synth.Case (or any object
    with .params, .elev, .rain, .reach, .mannings, .water_init)."""

    def __init__(self, case, max_bytes=0, prepare=True):
        self.lib = load_library()
        self.case = case
        self.p = case.params
        self.h = C.c_void_p()
        self._check(self.lib.hc_create(C.byref(self.p), max_bytes, C.byref(self.h)), "create")
        p = self.p
        elev = np.full((p.imax + 2, p.jmax + 2), -9999.0)
        elev[1:-1, 1:-1] = case.elev
        self.upload("elev", elev)
        if case.mannings is not None:
            m = np.zeros((p.imax + 2, p.jmax + 2))
            m[1:-1, 1:-1] = case.mannings
            self.upload("spat_var_mannings", m)
        if case.water_init is not None:
            w = np.zeros((p.imax + 2, p.jmax + 2))
            w[1:-1, 1:-1] = case.water_init
            self.upload("water_depth", w)
        r = np.ascontiguousarray(case.rain, dtype=np.float32)
        self._check(self.lib.hc_set_rain(self.h, r.ctypes.data, r.shape[0], r.shape[1]), "rain")
        for k, t in enumerate(case.reach):
            t = np.ascontiguousarray(t, dtype=np.float32)
            self._check(self.lib.hc_set_reach(self.h, k, t.ctypes.data, t.shape[0], t.shape[1]),
                        "reach")
        if prepare:
            self.prepare()

    def close(self):
        if self.h:
            self.lib.hc_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != 0:
            msg = self.lib.hc_last_error(self.h) if self.h else b""
            raise HCError("%s failed: %s %s" % (what, STATUS.get(st, st),
                                                (msg or b"").decode(errors="replace")))

    # ---- fields
    def upload(self, name, a):
        a = np.ascontiguousarray(a, dtype=field_dtype(name)).reshape(field_shape(self.p, name))
        self._check(self.lib.hc_upload(self.h, FIELD_ID[name], a.ctypes.data, a.nbytes),
                    "upload " + name)

    def field(self, name):
        a = np.empty(field_shape(self.p, name), dtype=field_dtype(name))
        self._check(self.lib.hc_download(self.h, FIELD_ID[name], a.ctypes.data, a.nbytes),
                    "download " + name)
        return a

    def scalars(self):
        s = hc_scalars()
        self._check(self.lib.hc_get_scalars(self.h, C.byref(s)), "get_scalars")
        return s

    def set_scalars(self, s):
        self._check(self.lib.hc_set_scalars(self.h, C.byref(s)), "set_scalars")

    # ---- members
    def prepare(self):
        self._check(self.lib.hc_prepare(self.h), "prepare")

    def set_maximum_timestep(self):
        self._check(self.lib.hc_set_maximum_timestep(self.h), "set_maximum_timestep")

    def flow_route(self):
        self._check(self.lib.hc_flow_route(self.h), "flow_route")

    def depth_update(self):
        self._check(self.lib.hc_depth_update(self.h), "depth_update")

    def scan_area(self):
        self._check(self.lib.hc_scan_area(self.h), "scan_area")

    def water_flux_out(self):
        self._check(self.lib.hc_water_flux_out(self.h), "water_flux_out")

    def erode(self, mult):
        t = C.c_double()
        self._check(self.lib.hc_erode(self.h, float(mult), C.byref(t)), "erode")
        return t.value

    def lateral_channel_erode(self):
        self._check(self.lib.hc_lateral_channel_erode(self.h), "lateral_channel_erode")

    def in_channel_landsliding(self):
        self._check(self.lib.hc_in_channel_landsliding(self.h), "in_channel_landsliding")

    def global_landsliding(self):
        """Returns the number of sweeps made."""
        n = C.c_int32()
        self._check(self.lib.hc_global_landsliding(self.h, C.byref(n)), "global_landsliding")
        return n.value

    def creep(self, time):
        self._check(self.lib.hc_creep(self.h, float(time)), "creep")

    # ---- whole iterations
    def run(self, n, flags=None, records=True):
        """Runs up to n iterations of the main loop; returns the per-iteration
        records as an (iterations, 14) float64 array (fields STEP_FIELDS)."""
        flags = self.case.flags if flags is None else flags
        rec = np.zeros((max(n, 1), len(STEP_FIELDS)), dtype=np.float64) if records else None
        done = C.c_int64()
        self._check(self.lib.hc_run(self.h, n, flags, rec.ctypes.data if records else None,
                                    C.byref(done)), "run")
        return rec[:done.value] if records else done.value

    def stream(self):
        return self.lib.hc_stream(self.h)

    # ---- water ledger
    def mass_balance(self):
        """{volume0, volume, inflow, outflow, lost, mask_edge} in m^3 since
        hc_prepare (or mass_reset); volume is measured now."""
        m = hc_mass()
        self._check(self.lib.hc_mass_balance(self.h, C.byref(m)), "mass_balance")
        return {k: getattr(m, k) for k, _ in hc_mass._fields_}

    def test_bounded_waits(self, spins, extra_arrivals=1):
        """Shortens the drainage sweep's device waits and makes them run out
        (spins 0: back to normal); see hc_test_bounded_waits."""
        self._check(self.lib.hc_test_bounded_waits(self.h, spins, extra_arrivals),
                    "test_bounded_waits")

    def autotune(self, force=False):
        """(launch shape in use, [ms per launch of each shape of the last
        tuning]) of k_flow_route; force=True times the shapes now."""
        shape = C.c_int32()
        ms = (C.c_double * 18)()
        self._check(self.lib.hc_autotune(self.h, 1 if force else 0, C.byref(shape), ms, 18),
                    "autotune")
        return shape.value, list(ms)

    def set_launch_shape(self, shape):
        """Fixes k_flow_route's launch shape (-1: the autotuner chooses)."""
        self._check(self.lib.hc_set_launch_shape(self.h, shape), "set_launch_shape")

    def mass_reset(self):
        self._check(self.lib.hc_mass_reset(self.h), "mass_reset")

    def bench_kernel(self, kernel, reps):
        """(mean ms per launch, wet cells) of one kernel, timed with CUDA
        events on the context's stream."""
        ms = C.c_double()
        wet = C.c_int64()
        self._check(self.lib.hc_bench_kernel(self.h, kernel.encode(), reps, C.byref(ms),
                                             C.byref(wet)), "bench_kernel")
        return ms.value, wet.value

    def counters(self):
        """(kernels launched, bytes host->device, bytes device->host) so far."""
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.lib.hc_get_counters(self.h, C.byref(a), C.byref(b), C.byref(c)),
                    "counters")
        return a.value, b.value, c.value

    # ---- snapshots
    def snapshot_begin(self, name, out):
        """Starts copying field `name` into `out` (a page-locked numpy array of
        the field's shape, e.g. from pinned_empty) while the run goes on;
        returns a handle for snapshot_end."""
        h = C.c_void_p()
        self._check(self.lib.hc_snapshot_begin(self.h, FIELD_ID[name], out.ctypes.data,
                                               out.nbytes, C.byref(h)), "snapshot_begin")
        return h

    def snapshot_end(self, handle):
        self._check(self.lib.hc_snapshot_end(handle), "snapshot_end")

    # ---- adjoint (hydro-only)
    ADJ_RECORD = 22

    def adj_forward(self, n, fixed=None, max_samples=100000):
        """Runs n iterations; returns (time-step record (n, 22), outlet Q at
        the first iteration of every simulated minute).  `fixed`: a record to
        impose instead of the adaptive time steps."""
        rec = np.zeros((n, self.ADJ_RECORD), dtype=np.float64)
        q = np.zeros(max_samples, dtype=np.float64)
        ns = C.c_int64()
        fx = None
        if fixed is not None:
            fx = np.ascontiguousarray(fixed, dtype=np.float64)
            assert fx.shape == (n, self.ADJ_RECORD)
        self._check(self.lib.hc_adj_forward(self.h, n, None if fx is None else fx.ctypes.data,
                                            rec.ctypes.data, q.ctypes.data, max_samples,
                                            C.byref(ns)), "adj_forward")
        return rec, q[:min(ns.value, max_samples)].copy()

    def adj_gradient(self, n, max_states, target, elev=False):
        """(loss, dL/dn per cell (imax+2, jmax+2), dL/drain (rain rows, cols),
        info) over n iterations from the current state, keeping at most
        max_states model states (binomial checkpointing); with elev=True also
        dL/d(elevation) per cell, as a fifth element.  info: forward_ms,
        reverse_ms, total_ms, segment, snapshots, advanced (iterations run
        again beyond the forward run and the segment replays)."""
        p = self.p
        t = np.ascontiguousarray(target, dtype=np.float64)
        gn = np.zeros((p.imax + 2, p.jmax + 2), dtype=np.float64)
        ge = np.zeros((p.imax + 2, p.jmax + 2), dtype=np.float64)
        gr = np.zeros(self.case.rain.shape, dtype=np.float64)
        loss = C.c_double()
        ms = (C.c_double * 8)()
        self._check(self.lib.hc_adj_gradient(self.h, n, max_states, t.ctypes.data, len(t),
                                             C.byref(loss), gn.ctypes.data, gr.ctypes.data,
                                             ge.ctypes.data, ms), "adj_gradient")
        info = dict(zip(("forward_ms", "reverse_ms", "total_ms", "segment", "snapshots",
                         "advanced", "replay_ms", "adjoint_iterations_ms"), list(ms)))
        if elev:
            return loss.value, gn, gr, info, ge
        return loss.value, gn, gr, info

    RUN_STATS = ["chunks", "erode_retry", "lateral", "creep", "global_slide", "drainage",
                 "drainage_sort", "drainage_sweep", "drainage_levels", "idle_iters",
                 "drainage_host_sort", "wet_cell_steps"]

    def run_stats(self):
        """{kind: (count, host ms)} of hc_run's host-side work so far."""
        n = len(self.RUN_STATS)
        cnt = (C.c_int64 * n)()
        ms = (C.c_double * n)()
        self._check(self.lib.hc_get_run_stats(self.h, cnt, ms, n), "run_stats")
        return {k: (cnt[i], ms[i]) for i, k in enumerate(self.RUN_STATS)}

    PHASES = ["control_inputs", "flow_route", "depth_update", "scan_area", "entrain_passes",
              "apply_lateral_edge", "lateral3", "water_flux_out", "slide_3"]

    def profile_iteration(self, flags=None):
        """{phase: ms} for one iteration run phase by phase with CUDA events."""
        flags = self.case.flags if flags is None else flags
        ms = (C.c_double * 9)()
        self._check(self.lib.hc_profile_iteration(self.h, flags, ms), "profile_iteration")
        return dict(zip(self.PHASES, list(ms)))


def run_ensemble(models, n, flags=0):
    """Runs up to n iterations of every model at once (hc_run_ensemble);
    returns the iteration counts."""
    lib = load_library()
    m = len(models)
    arr = (C.c_void_p * m)(*[mod.h.value for mod in models])
    done = (C.c_int64 * m)()
    st = lib.hc_run_ensemble(arr, m, n, flags, done)
    if st != 0:
        msgs = [(mod.lib.hc_last_error(mod.h) or b"").decode() for mod in models]
        raise HCError("run_ensemble failed: %s %s" % (STATUS.get(st, st),
                                                    "; ".join(x for x in msgs if x)))
    return list(done)
