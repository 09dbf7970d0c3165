"""ctypes mirror of include/hc_gpu.h (the C ABI of libhc_gpu).

Field layouts, defaults and names follow the reference's LSDCatchmentModel
(include/catchmentmodel/LSDCatchmentModel.hpp:437-568 for the defaults).
"""
import ctypes as C

HC_G_MAX = 10
HC_NSTRATA = 10
HC_MAX_RF = 16
HC_MAX_POINTS = 3

HC_RUN_LATERAL = 1
HC_RUN_NOHILL = 2

STATUS = {0: "HC_OK", 1: "HC_ERR_ARG", 2: "HC_ERR_CUDA", 3: "HC_ERR_NONFINITE",
          4: "HC_ERR_TIMEOUT", 5: "HC_ERR_NOMEM", 6: "HC_ERR_STATE",
          7: "HC_ERR_UNSUPPORTED"}


class hc_params(C.Structure):
    _fields_ = [
        ("imax", C.c_int32), ("jmax", C.c_int32), ("DX", C.c_double),
        ("courant_number", C.c_double), ("froude_limit", C.c_double),
        ("mannings", C.c_double), ("hflow_threshold", C.c_double),
        ("edgeslope", C.c_double), ("water_depth_erosion_threshold", C.c_double),
        ("in_out_difference_allowed", C.c_double), ("max_time_step", C.c_int32),
        ("spatially_var_mannings", C.c_int32), ("ERODEFACTOR", C.c_double),
        ("maxcycle", C.c_int32),
        ("rain_data_time_step", C.c_double), ("rfnum", C.c_int32), ("M", C.c_double),
        ("rain_factor", C.c_double), ("baseflow", C.c_double), ("MIN_Q", C.c_double),
        ("MIN_Q_MAXVAL", C.c_double),
        ("reach_mode", C.c_int32), ("number_of_points", C.c_int32),
        ("inpoints", (C.c_int32 * 2) * HC_MAX_POINTS),
        ("reach_input_data_timestep", C.c_int32), ("div_inputs", C.c_int32),
        ("hydro_only", C.c_int32), ("wilcock", C.c_int32), ("einstein", C.c_int32),
        ("active", C.c_double), ("max_vel", C.c_double), ("Csuspmax", C.c_double),
        ("bedrock_erosion_threshold", C.c_double), ("bedrock_erosion_rate", C.c_double),
        ("vegTauCrit", C.c_double), ("veg_lat_restriction", C.c_double),
        ("lateral_constant", C.c_double), ("chann_lateral_erosion", C.c_double),
        ("failureangle", C.c_double), ("CREEP_RATE", C.c_double),
        ("d", C.c_double * HC_G_MAX), ("dprop", C.c_double * (HC_G_MAX + 1)),
        ("fallVelocity", C.c_double * (HC_G_MAX + 1)),
        ("isSuspended", C.c_int32 * (HC_G_MAX + 1)), ("vegetation_on", C.c_int32),
        ("edge_smoothing_passes", C.c_double), ("downstream_shift", C.c_double),
        ("lateral_cross_channel_smoothing", C.c_double),
        ("scan_area_interval_iter", C.c_int32),
        ("in_channel_landslide_iter_interval", C.c_int32),
        ("creep_time_interval", C.c_int32), ("global_landsliding_interval", C.c_int32),
        ("creep_coeff", C.c_double), ("LIMIT", C.c_int32),
        ("spatially_complex_rainfall", C.c_int32),
    ]


_RF = C.c_double * (HC_MAX_RF + 1)


class hc_scalars(C.Structure):
    _fields_ = [
        ("cycle", C.c_double), ("previous", C.c_double), ("time_step", C.c_double),
        ("maxdepth", C.c_double), ("waterinput", C.c_double), ("waterOut", C.c_double),
        ("input_output_difference", C.c_double), ("temptot", C.c_double),
        ("counter", C.c_double), ("erode_call", C.c_double), ("erode_mult", C.c_double),
        ("lateralcounter", C.c_double), ("time_1", C.c_double), ("baseflow", C.c_double),
        ("grain_array_tot", C.c_double), ("sediQ", C.c_double),
        ("globalsediq", C.c_double), ("tempbmax", C.c_double),
        ("creep_time", C.c_double), ("creep_time2", C.c_double),
        ("sum_grain", C.c_double * (HC_G_MAX + 1)),
        ("j", _RF), ("jo", _RF), ("j_mean", _RF), ("old_j_mean", _RF),
        ("new_j_mean", _RF), ("nActualGridCells", _RF),
        ("catchment_input_counter", _RF), ("totalinputpoints", C.c_double),
        ("flow_timestep", C.c_double), ("stop_flag", C.c_double),
    ]


class hc_step_record(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "counter", "cycle", "time_step", "maxdepth", "waterOut", "waterinput",
        "erode_mult", "sediQ", "globalsediq", "baseflow", "vol_in", "vol_out", "vol_mask", "volume")]


STEP_FIELDS = [f[0] for f in hc_step_record._fields_]
# the fields the reference harness (oracle/ref_harness.cpp) records
REF_STEP_FIELDS = STEP_FIELDS[:10]


class hc_mass(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("volume0", "volume", "inflow", "outflow", "lost",
                                             "mask_edge")]

# hc_field enum, in declaration order
FIELDS = ["elev", "water_depth", "qx", "qy", "qxs", "qys", "Vsusptot", "Vel", "Tau",
          "bedrock", "spat_var_mannings", "area", "ss", "vel_dir", "sr", "sl", "su",
          "sd", "index", "grain", "strata", "down_scan", "edge", "veg", "rfarea",
          "inputpointsarray"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}


def field_shape(p, name):
    """numpy shape of a field in the reference (TNT) layout."""
    i2, j2 = p.imax + 2, p.jmax + 2
    nrec = (i2 * j2) // max(1, p.LIMIT)
    if name in ("vel_dir",):
        return (i2, j2, 9)
    if name in ("sr", "sl", "su", "sd"):
        return (i2, j2, 10)
    if name == "grain":
        return (nrec, 11)
    if name == "strata":
        return (nrec, 10, 11)
    if name == "down_scan":
        return (j2, i2)
    if name in ("edge",):
        return (p.imax + 1, p.jmax + 1)
    if name == "veg":
        return (p.imax + 1, p.jmax + 1, 4)
    return (i2, j2)


def field_dtype(name):
    import numpy as np
    if name in ("index", "down_scan", "rfarea"):
        return np.int32
    if name == "inputpointsarray":
        return np.uint8
    return np.float64


def default_params(imax, jmax, DX):
    """The reference's member initialisers (LSDCatchmentModel.hpp:437-568)
    and the driver constants of main.cpp:127-132."""
    p = hc_params()
    p.imax, p.jmax, p.DX = imax, jmax, DX
    p.courant_number = 0.7
    p.froude_limit = 0.8
    p.mannings = 0.04
    p.hflow_threshold = 0.00001
    p.edgeslope = 0.001
    p.water_depth_erosion_threshold = 0.01
    p.in_out_difference_allowed = 0.0
    p.max_time_step = 0
    p.spatially_var_mannings = 0
    p.ERODEFACTOR = 0.05
    p.maxcycle = 1000
    p.rain_data_time_step = 60
    p.rfnum = 1
    p.M = 0.005
    p.rain_factor = 1
    p.baseflow = 0.00000005
    p.MIN_Q = 0.01
    p.MIN_Q_MAXVAL = 1000.0
    p.reach_mode = 0
    p.number_of_points = 0
    p.reach_input_data_timestep = 60
    p.div_inputs = 1
    p.hydro_only = 0
    p.wilcock = 0
    p.einstein = 0
    p.active = 0.2
    p.max_vel = 5
    p.Csuspmax = 0.05
    p.bedrock_erosion_threshold = 0
    p.bedrock_erosion_rate = 0
    p.vegTauCrit = 100
    p.veg_lat_restriction = 0.1
    p.lateral_constant = 0.0000002
    p.chann_lateral_erosion = 20.0
    p.failureangle = 45
    p.CREEP_RATE = 0.0025
    for n, v in enumerate([0.0, 0.000065, 0.001, 0.002, 0.004, 0.008, 0.016, 0.032,
                           0.064, 0.128]):
        p.d[n] = v
    for n, v in enumerate([0.0, 0.05, 0.05, 0.15, 0.225, 0.25, 0.1, 0.075, 0.05, 0.05,
                           0.0]):
        p.dprop[n] = v
    for n, v in enumerate([0.0, 0.033, 0.109, 0.164, 0.237, 0.338, 0.479, 0.678, 0.959,
                           1.357, 0.0]):
        p.fallVelocity[n] = v
    for n in range(HC_G_MAX + 1):
        p.isSuspended[n] = 1 if n == 1 else 0
    p.vegetation_on = 0
    p.edge_smoothing_passes = 100.0
    p.downstream_shift = 5.0
    p.lateral_cross_channel_smoothing = 0.0001
    p.scan_area_interval_iter = 5
    p.in_channel_landslide_iter_interval = 10
    p.creep_time_interval = 14400
    p.global_landsliding_interval = 1440
    p.creep_coeff = 0.028
    p.LIMIT = 1
    return p


def params_to_dict(p):
    out = {}
    for name, _ in p._fields_:
        v = getattr(p, name)
        if hasattr(v, "__len__"):
            v = [list(x) if hasattr(x, "__len__") else x for x in v]
        out[name] = v
    return out


def params_from_dict(d):
    p = hc_params()
    for name, _ in p._fields_:
        if name not in d:
            continue
        v = d[name]
        if name == "inpoints":
            for a in range(HC_MAX_POINTS):
                for b in range(2):
                    p.inpoints[a][b] = int(v[a][b])
        elif isinstance(v, (list, tuple)):
            arr = getattr(p, name)
            for k, x in enumerate(v):
                arr[k] = x
        else:
            setattr(p, name, v)
    return p
