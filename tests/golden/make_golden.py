"""Generates the committed golden fixtures of tests/golden/ (run here, where
the reference checkout exists; the fixtures travel, the reference does not).

1. boscastle_kga.npz - the reference's own known-good answers
   (test/known_good_answers/, checked by test/basic_kga_tests.py) with the
   inputs that produce them: the Boscastle 50 m DEM (normal and flipped
   left-right), the rain table, the model parameters as the reference reads
   them from its .params file, the WaterDepths3360 rasters and the hydrograph
   column of the .dat files.
2. ref_<case>.npz - final state and per-iteration records of the unmodified
   reference sources (oracle/_ref/ref_harness) on small seeded synthetic cases.

Usage:  python tests/golden/make_golden.py --reference <reference checkout>
        (or HC_REFERENCE set in the environment)
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "hail-caesar_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import hc_abi  # noqa: E402
import synth  # noqa: E402

# --------------------------------------------------------------- .params
# keys -> (hc_params field, converter), as LSDCatchmentModel::initialise_variables
# (LSDCatchmentModel.cpp:842-1600) assigns them
KEYS = {
    "max_time_step": ("max_time_step", int),
    "max_run_duration": ("maxcycle", int),
    "memory_limit": ("LIMIT", int),
    "max_tau_velocity": ("max_vel", float),
    "active_layer_thickness": ("active", float),
    "chann_lateral_erosion": ("chann_lateral_erosion", float),
    "erosion_limit": ("ERODEFACTOR", float),
    "edge_smoothing_passes": ("edge_smoothing_passes", float),
    "lateral_erosion_const": ("lateral_constant", float),
    "downstream_cell_shift": ("downstream_shift", float),
    "lateral_cross_chan_smoothing": ("lateral_cross_channel_smoothing", float),
    "topmodel_m_value": ("M", float),
    "num_unique_rain_cells": ("rfnum", int),
    "rain_data_time_step": ("rain_data_time_step", float),
    "in_out_difference": ("in_out_difference_allowed", float),
    "min_q_for_depth_calc": ("MIN_Q", float),
    "max_q_for_depth_calc": ("MIN_Q_MAXVAL", float),
    "hflow_threshold": ("hflow_threshold", float),
    # the reference assigns this key to hflow_threshold (:1318-1321)
    "water_depth_erosion_threshold": ("hflow_threshold", float),
    "slope_on_edge_cell": ("edgeslope", float),
    "courant_number": ("courant_number", float),
    "froude_num_limit": ("froude_limit", float),
    "mannings_n": ("mannings", float),
    "vegetation_crit_shear": ("vegTauCrit", float),
    "veg_erosion_prop": ("veg_lat_restriction", float),
    "creep_rate": ("CREEP_RATE", float),
    "slope_failure_thresh": ("failureangle", float),
}


def parse_params(path):
    """key: value pairs in file order (LSDUtils.cpp:12-77 semantics: the
    first token after ':' up to whitespace, '#' starts a comment)."""
    out = []
    for line in open(path):
        line = line.split("#", 1)[0]
        if ":" not in line:
            continue
        k, v = line.split(":", 1)
        v = v.strip().split()
        if not v:
            continue
        out.append((k.strip().lower(), v[0]))
    return out


def params_from_file(path, imax, jmax, DX):
    p = hc_abi.default_params(imax, jmax, DX)
    flags = {}
    for k, v in parse_params(path):
        if k in KEYS:
            name, conv = KEYS[k]
            setattr(p, name, conv(float(v)) if conv is int else conv(v))
        elif k == "transport_law":
            p.wilcock, p.einstein = (1, 0) if v == "wilcock" else (0, 1)
        elif k == "hydro_model_only":
            p.hydro_only = 1 if v == "yes" else 0
        elif k in ("spatial_var_rain", "timeseries_save_interval", "raster_output_interval"):
            flags[k] = v
    if flags.get("spatial_var_rain", "no") != "yes":
        p.rfnum = 1  # :1602-1608
    if p.rain_data_time_step < 1:  # initialise_arrays :1680-1684
        p.rain_data_time_step = 1
    if p.max_time_step // 60 > p.rain_data_time_step:
        p.max_time_step = int(p.rain_data_time_step) * 60
    return p, flags


def read_asc(path):
    with open(path) as f:
        hdr = {}
        for _ in range(6):
            k, v = f.readline().split()
            hdr[k.lower()] = float(v)
        data = np.loadtxt(f)
    return hdr, data


def read_rain(path):
    rows = [[np.float32(x) for x in line.split()] for line in open(path) if line.strip()]
    w = max(len(r) for r in rows)
    t = np.zeros((len(rows), w), dtype=np.float32)
    for i, r in enumerate(rows):
        t[i, :len(r)] = r
    return t


def make_boscastle(ref):
    base = os.path.join(ref, "test", "input_data", "boscastle", "boscastle_input_data")
    kga = os.path.join(ref, "test", "known_good_answers")
    out = {}
    for tag, dem, params, kdir, dat in [
        ("normal", "boscastle_square_50m.asc", "boscastle_test_72hr_50m_u.params",
         "boscastle50m_72hr_u", "boscastle_50m_72hr_u.dat"),
        ("flipped", "boscastle_flipped_lr_50m.asc", "boscastle_test_72hr_50m_u_flipped_lr.params",
         "boscastle50m_72hr_u_flipped_lr", "boscastle_50m_72hr_u_flipped_lr.dat")]:
        hdr, z = read_asc(os.path.join(base, dem))
        imax, jmax = z.shape
        p, flags = params_from_file(os.path.join(base, params), imax, jmax, hdr["cellsize"])
        _, wd = read_asc(os.path.join(kga, kdir, "WaterDepths3360.asc"))
        q = np.loadtxt(os.path.join(kga, kdir, dat), usecols=1)
        out[tag + "_elev"] = z
        out[tag + "_params"] = np.array(json.dumps(hc_abi.params_to_dict(p)))
        out[tag + "_wd3360"] = wd
        out[tag + "_hydrograph"] = q
        out[tag + "_interval"] = np.array(float(flags.get("timeseries_save_interval", 60)))
        out[tag + "_raster_interval"] = np.array(float(flags.get("raster_output_interval", 1000)))
    out["rain"] = read_rain(os.path.join(base, "boscastle_72hr_rain_u.txt"))
    np.savez_compressed(os.path.join(HERE, "boscastle_kga.npz"), **out)


# --------------------------------------------------------------- synthetic
def golden_cases():
    """name -> (case, iterations).  Small enough for the oracle in seconds."""
    return {
        "reach_hydro": (synth.reach_case(imax=60, jmax=24, DX=10.0, hours=24, hydro_only=True), 2500),
        "reach_erosion": (synth.reach_case(imax=60, jmax=24, DX=10.0, hours=24), 2500),
        "catchment_hydro": (synth.catchment_case(n=40, DX=20.0, hours=72, relief=60.0,
                                                 hydro_only=True, lateral=False), 6000),
        "catchment_lateral": (synth.catchment_case(n=33, DX=20.0, hours=72, relief=60.0,
                                                   lateral=True), 12000),
        "catchment_odd": (synth.catchment_case(n=29, jmax=18, DX=10.0, hours=72, relief=40.0,
                                               lateral=False), 8000),
    }


SAVE = ["elev", "water_depth", "qx", "qy", "qxs", "qys", "Vsusptot", "Vel", "Tau", "index",
        "down_scan", "vel_dir", "grain", "strata", "ss", "edge", "area"]


def make_synthetic():
    import oracle
    for name, (case, n) in golden_cases().items():
        st, rec = oracle.run_reference(case, n)
        keep = {k: st[k] for k in SAVE if k in st}
        if "grain" in keep:
            # only the rows in use (index values 2..grain_array_tot)
            used = int(st["grain_array_tot"]) + 1
            keep["grain"] = keep["grain"][:used]
            keep["strata"] = keep["strata"][:used]
        keep["records"] = rec
        keep["iterations"] = np.array(n)
        for s in ("cycle", "time_step", "grain_array_tot", "sediQ", "globalsediq", "baseflow",
                  "totalinputpoints", "erode_mult", "erode_call"):
            keep["s_" + s] = np.array(st[s])
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % name), **keep)
        print(name, {k: v.shape for k, v in keep.items() if hasattr(v, "shape") and v.ndim})


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("HC_REFERENCE"))
    a = ap.parse_args()
    if not a.reference:
        ap.error("name the reference checkout: --reference or HC_REFERENCE")
    os.environ["HC_REFERENCE"] = a.reference
    make_boscastle(a.reference)
    make_synthetic()
