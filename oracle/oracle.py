"""Python side of the oracle (test infrastructure).

* `Oracle`      ctypes wrapper of liboracle.so, the CPU restatement
                (hc_oracle.cpp) of the reference's per-step path.
* `run_reference` writes a case as the reference's own input files
                (.params, .asc rasters, rain and reach tables) and runs
                oracle/_ref/ref_harness, the unmodified reference sources,
                returning its in-memory state.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the product never does.
"""
import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(os.path.dirname(HERE), "hail-caesar_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

from hc_abi import (hc_params, STEP_FIELDS, field_shape, field_dtype,  # noqa: E402
                    HC_RUN_LATERAL, HC_RUN_NOHILL)

REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")
REF_HARNESS_OMP = os.path.join(HERE, "_ref", "ref_harness_omp")


class _Rec(C.Structure):
    _fields_ = [(n, C.c_double) for n in STEP_FIELDS]


def build(quiet=True):
    """Builds liboracle(.so, _omp.so); also the reference harness when the
    environment's HC_REFERENCE names the reference checkout."""
    targets = ["oracle"]
    ref = os.environ.get("HC_REFERENCE", "")
    if ref and os.path.isdir(os.path.join(ref, "src", "catchmentmodel")):
        targets.append("ref")
    cmd = ["make", "-s", "-C", HERE, "-j8"] + targets
    if "ref" in targets:
        cmd.append("REF=" + ref)
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL if quiet else None)


_LIBS = {}


def _lib(omp=False):
    name = "liboracle_omp.so" if omp else "liboracle.so"
    if name not in _LIBS:
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        lib.hco_create.restype = C.c_void_p
        lib.hco_create.argtypes = [C.POINTER(hc_params)]
        lib.hco_destroy.argtypes = [C.c_void_p]
        lib.hco_field.restype = C.c_void_p
        lib.hco_field.argtypes = [C.c_void_p, C.c_char_p]
        lib.hco_field_size.restype = C.c_int64
        lib.hco_field_size.argtypes = [C.c_void_p, C.c_char_p]
        lib.hco_field_elsize.restype = C.c_int
        lib.hco_field_elsize.argtypes = [C.c_void_p, C.c_char_p]
        lib.hco_get_scalar.restype = C.c_double
        lib.hco_get_scalar.argtypes = [C.c_void_p, C.c_char_p]
        lib.hco_set_scalar.restype = C.c_int
        lib.hco_set_scalar.argtypes = [C.c_void_p, C.c_char_p, C.c_double]
        lib.hco_set_rain.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        lib.hco_set_reach.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int]
        lib.hco_prepare.argtypes = [C.c_void_p]
        lib.hco_resume.argtypes = [C.c_void_p]
        lib.hco_iterate.restype = C.c_long
        lib.hco_iterate.argtypes = [C.c_void_p, C.c_long, C.c_int, C.c_void_p]
        lib.hco_erode.restype = C.c_double
        lib.hco_erode.argtypes = [C.c_void_p, C.c_double]
        for f in ("hco_flow_route", "hco_depth_update", "hco_scan_area",
                  "hco_water_flux_out", "hco_lateral_channel_erode",
                  "hco_in_channel_landsliding", "hco_global_landsliding",
                  "hco_set_maximum_timestep"):
            getattr(lib, f).argtypes = [C.c_void_p]
        lib.hco_creep.argtypes = [C.c_void_p, C.c_double]
        lib.hco_sort_perm.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
        lib.hco_get_flow_timestep.restype = C.c_double
        lib.hco_get_flow_timestep.argtypes = [C.c_void_p]
        _LIBS[name] = lib
    return _LIBS[name]


class Oracle:
    """The CPU restatement holding one model state."""

    def __init__(self, case, omp=False):
        self.case = case
        self.p = case.params
        self.lib = _lib(omp)
        self.h = self.lib.hco_create(C.byref(self.p))
        p = self.p
        self.field("elev")[1:-1, 1:-1] = case.elev
        if case.mannings is not None:
            self.field("spat_var_mannings")[1:-1, 1:-1] = case.mannings
        if case.water_init is not None:
            self.field("water_depth")[1:-1, 1:-1] = case.water_init
        r = np.ascontiguousarray(case.rain, dtype=np.float32)
        self.lib.hco_set_rain(self.h, r.ctypes.data, r.shape[0], r.shape[1])
        for k, t in enumerate(case.reach):
            t = np.ascontiguousarray(t, dtype=np.float32)
            self.lib.hco_set_reach(self.h, k, t.ctypes.data, t.shape[0], t.shape[1])
        self._keep = (r, [np.ascontiguousarray(t, np.float32) for t in case.reach])
        self.prepared = False

    def __del__(self):
        try:
            self.lib.hco_destroy(self.h)
        except Exception:
            pass

    def field(self, name):
        """numpy view (reference layout) of a state field."""
        n = self.lib.hco_field_size(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        ptr = self.lib.hco_field(self.h, name.encode())
        dt = field_dtype(name)
        if name in ("cin_x", "cin_y"):
            shape = (n,)
        else:
            shape = field_shape(self.p, name)
        buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(ptr)
        return np.frombuffer(buf, dtype=dt).reshape(shape)

    def scalar(self, name):
        return self.lib.hco_get_scalar(self.h, name.encode())

    def set_scalar(self, name, v):
        if self.lib.hco_set_scalar(self.h, name.encode(), float(v)) != 0:
            raise KeyError(name)

    def prepare(self):
        self.lib.hco_prepare(self.h)
        self.prepared = True

    def iterate(self, n, flags=None):
        if not self.prepared:
            self.prepare()
        flags = self.case.flags if flags is None else flags
        cap = n if n >= 0 else 10_000_000
        rec = np.zeros((cap, len(STEP_FIELDS)), dtype=np.float64)
        done = self.lib.hco_iterate(self.h, n, flags, rec.ctypes.data)
        if self.scalar("grain_full"):
            raise RuntimeError("grain records beyond the N2/LIMIT rows the reference allocates")
        return rec[:done]

    def load_from(self, model):
        """Copies the whole state of a GPU model (hc.Model) into this oracle
        and continues from it (fields in the reference layout, scalars, then
        hco_resume)."""
        names = ["elev", "water_depth", "qx", "qy", "qxs", "qys", "Vsusptot", "Vel", "Tau",
                 "bedrock", "spat_var_mannings", "area", "index", "down_scan", "edge", "veg",
                 "rfarea", "vel_dir"]
        if not self.p.hydro_only:
            names += ["ss", "sr", "sl", "su", "sd", "grain", "strata"]
        for k in names:
            self.field(k)[...] = model.field(k)
        s = model.scalars()
        for k in ("cycle", "previous", "time_step", "maxdepth", "waterinput", "waterOut",
                  "counter", "erode_call", "erode_mult", "lateralcounter", "time_1", "baseflow",
                  "grain_array_tot", "sediQ", "globalsediq", "creep_time", "creep_time2"):
            self.set_scalar(k, getattr(s, k))
        for n in range(1, self.p.rfnum + 1):
            self.set_scalar("j_mean%d" % n, s.j_mean[n])
        for n in range(1, 11):
            self.set_scalar("sum_grain%d" % n, s.sum_grain[n])
        self.lib.hco_resume(self.h)
        self.prepared = True

    def state(self, names=None):
        names = names or ["elev", "water_depth", "qx", "qy", "qxs", "qys", "Vsusptot",
                          "Vel", "Tau", "index", "down_scan", "vel_dir"]
        return {k: self.field(k).copy() for k in names}


# ---------------------------------------------------------------- reference
def _fmt(v):
    return repr(float(v))


def write_asc(path, a, DX):
    imax, jmax = a.shape
    with open(path, "w") as f:
        f.write("ncols %d\nnrows %d\nxllcorner 0\nyllcorner 0\ncellsize %s\n"
                "NODATA_value -9999\n" % (jmax, imax, _fmt(DX)))
        for row in a:
            f.write(" ".join(_fmt(v) for v in row))
            f.write("\n")


def write_table(path, t):
    with open(path, "w") as f:
        for row in t:
            f.write(" ".join(repr(float(np.float32(v))) for v in row))
            f.write("\n")


def write_reference_inputs(case, d):
    """The case as the reference's own input files in directory d."""
    p = case.params
    write_asc(os.path.join(d, "dem.asc"), case.elev, p.DX)
    rain_on = case.rain is not None and not case.reach
    if rain_on:
        write_table(os.path.join(d, "rain.txt"), case.rain)
    for k, t in enumerate(case.reach):
        write_table(os.path.join(d, "reach%d.txt" % (k + 1)), t)
    if case.mannings is not None:
        write_asc(os.path.join(d, "mannings.asc"), case.mannings, p.DX)
    kv = [
        ("read_fname", "dem"), ("dem_read_extension", "asc"), ("dem_write_extension", "asc"),
        ("read_path", d + "/"), ("write_path", d + "/"), ("write_fname", "ts.dat"),
        ("timeseries_save_interval", "60"),
        ("max_time_step", str(p.max_time_step)), ("min_time_step", "0"),
        ("max_run_duration", str(p.maxcycle)), ("memory_limit", str(p.LIMIT)),
        ("transport_law", "wilcock" if p.wilcock else "einstein"),
        ("max_tau_velocity", _fmt(p.max_vel)), ("active_layer_thickness", _fmt(p.active)),
        ("chann_lateral_erosion", _fmt(p.chann_lateral_erosion)),
        ("erosion_limit", _fmt(p.ERODEFACTOR)), ("suspended_sediment_on", "yes"),
        ("read_in_graindata_from_file", "no"), ("bedrock_layer_on", "no"),
        ("lateral_erosion_on", "no"), ("lateral_erosion_const", _fmt(p.lateral_constant)),
        ("edge_smoothing_passes", _fmt(p.edge_smoothing_passes)),
        ("downstream_cell_shift", _fmt(p.downstream_shift)),
        ("lateral_cross_chan_smoothing", _fmt(p.lateral_cross_channel_smoothing)),
        ("hydro_model_only", "yes" if p.hydro_only else "no"),
        ("topmodel_m_value", _fmt(p.M)), ("in_out_difference", _fmt(p.in_out_difference_allowed)),
        ("min_q_for_depth_calc", _fmt(p.MIN_Q)), ("max_q_for_depth_calc", _fmt(p.MIN_Q_MAXVAL)),
        ("hflow_threshold", _fmt(p.hflow_threshold)), ("slope_on_edge_cell", _fmt(p.edgeslope)),
        ("evaporation_rate", "0.0"), ("courant_number", _fmt(p.courant_number)),
        ("froude_num_limit", _fmt(p.froude_limit)), ("mannings_n", _fmt(p.mannings)),
        ("rainfall_data_on", "yes" if rain_on else "no"),
        ("rain_data_time_step", _fmt(p.rain_data_time_step)),
        ("spatial_var_rain", "no"), ("num_unique_rain_cells", str(p.rfnum)),
        ("spatially_complex_rainfall_on", "yes" if p.spatially_complex_rainfall else "no"),
        ("vegetation_on", "no"), ("grass_grow_rate", "0.0"),
        ("vegetation_crit_shear", _fmt(p.vegTauCrit)),
        ("veg_erosion_prop", _fmt(p.veg_lat_restriction)),
        ("creep_rate", _fmt(p.CREEP_RATE)), ("slope_failure_thresh", _fmt(p.failureangle)),
        ("raster_output_interval", "100000000"),
        ("write_waterdepth_file", "no"), ("write_elev_file", "no"),
        ("write_grainsize_file", "no"), ("write_elevdiff_file", "no"),
        ("debug_print_cycle", "no"),
    ]
    if p.spatially_var_mannings:
        kv += [("spatially_variable_mannings_on", "yes"),
               ("spatial_mannings_dem_file", "mannings.asc")]
    if rain_on:
        kv.append(("rainfall_data_file", "rain.txt"))
    if p.reach_mode:
        kv += [("reach_mode", "yes"), ("reach_input_data_timestep", str(p.reach_input_data_timestep)),
               ("divide_inputs_by", str(p.div_inputs))]
        for k in range(p.number_of_points):
            kv += [("reach%d_input_on" % (k + 1), "yes"),
                   ("reach%d_input_file" % (k + 1), "reach%d.txt" % (k + 1)),
                   ("reach%d_x" % (k + 1), str(p.inpoints[k][0])),
                   ("reach%d_y" % (k + 1), str(p.inpoints[k][1]))]
    with open(os.path.join(d, "case.params"), "w") as f:
        for k, v in kv:
            f.write("%s: %s\n" % (k, v))
    with open(os.path.join(d, "overrides.txt"), "w") as f:
        f.write("d " + " ".join(_fmt(p.d[n]) for n in range(1, 10)) + "\n")
        f.write("dprop " + " ".join(_fmt(p.dprop[n]) for n in range(11)) + "\n")
        f.write("fallvel " + " ".join(_fmt(p.fallVelocity[n]) for n in range(10)) + "\n")


def read_dump(path):
    out = {}
    codes = {"d": np.float64, "i": np.int32}
    with open(path, "rb") as f:
        while True:
            nm = f.read(32)
            if len(nm) < 32:
                break
            name = nm.split(b"\0")[0].decode()
            code = f.read(1).decode()
            count = int(np.frombuffer(f.read(8), np.uint64)[0])
            dt = codes[code]
            a = np.frombuffer(f.read(count * np.dtype(dt).itemsize), dtype=dt)
            out[name] = a if count > 1 else a[0]
    return out


def run_reference(case, iters, flags=None, omp=False, workdir=None, threads=None):
    """Runs the unmodified reference (oracle/_ref/ref_harness) on the case.
    Returns (state dict with arrays reshaped to the reference layout,
    step records array)."""
    exe = REF_HARNESS_OMP if omp else REF_HARNESS
    if not os.path.exists(exe):
        raise FileNotFoundError("reference harness not built: " + exe)
    flags = case.flags if flags is None else flags
    own = workdir is None
    d = workdir or tempfile.mkdtemp(prefix="hcref_")
    write_reference_inputs(case, d)
    args = [exe, d + "/", "case.params", str(iters), os.path.join(d, "out.bin"),
            os.path.join(d, "overrides.txt")]
    if flags & HC_RUN_LATERAL:
        args.append("lateral")
    if flags & HC_RUN_NOHILL:
        args.append("nohill")
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE,
                   env=env)
    st = read_dump(os.path.join(d, "out.bin"))
    rec = np.fromfile(os.path.join(d, "out.bin.steps"), dtype=np.float64).reshape(-1, 10)
    p = case.params
    for k, v in list(st.items()):
        if isinstance(v, np.ndarray):
            try:
                st[k] = v.reshape(field_shape(p, k))
            except ValueError:
                pass
    if own:
        import shutil
        shutil.rmtree(d, ignore_errors=True)
    return st, rec
