"""Benchmark: cell-steps/s of HAIL-CAESAR's per-timestep raster path on GB300.

One step = one iteration of the reference's main loop (src/main.cpp:139-204):
inputs, flow_route, depth_update, the Courant dt, scan_area, erosion/deposition
with grain sorting, lateral3, water_flux_out and slide_3, on one batch of
synthetic input already resident in HBM.

Workloads (seeded synthetic inputs with the benchmark configurations' shapes):
  catchment2000  (default) catchment mode, 2000 x 2000 cells at 20 m, fractal
                 DEM with 300 m relief pit-filled to one outlet edge,
                 gamma rain + 60 mm/h storm from 60 min, per-cell Manning's n,
                 Einstein transport, lateral3 and slide_3 on; 500 iterations
                 of spin-up (to simulated minute 117.6, inside the storm)
  flow8192       flow-only 8192 x 8192 at 5 m, 30 mm/h rain, erosion off
  reach          reach mode 300 x 100 at 10 m, Wilcock-Crowe

Both arms spin up by the same number of iterations, so they time the same
iterations of the same (deterministic) run.  --impl gb300 (default) times
libhc_gpu; --impl reference times the CPU implementation of the path (the
oracle port, OpenMP over the reference's own column loops) on the host cores.

Replicas only: under torchrun each rank runs its own model on its own GPU;
no data moves between ranks; value = all ranks' cell-steps / max rank time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

# hc_run_ensemble keeps one stream per member in flight: let the device give
# them as many hardware queues as it has (the default 8 would make
# unrelated members' kernels wait on one another).  Read when the CUDA
# context is created, so before torch initialises it.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "hail-caesar_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

import synth  # noqa: E402
from hc_abi import HC_RUN_LATERAL  # noqa: E402

METRIC = "cell-steps/s on 1 GB300 (plain vs batched ensemble); adjoint/forward cost"
UNIT = "cell-steps/s"
DATA = "synthetic (seeded generators, hail-caesar_gb300/synth.py)"


def workload_config(args, case, desc, spin_its):
    """The `config` of both arms' lines (identical for the same workload)."""
    return {"workload": args.workload, "description": desc, "cells": case.cells,
            "spinup_iterations": spin_its, "timed_iterations": args.steps,
            "parallelism": "replicas x%d" % args.gpus,
            "l2": "inputs larger than L2 (model state several GB)"}


def make_workload(name, size=0):
    """(case, spin-up iterations, description)."""
    if name == "catchment2000":
        n = size or 2000
        case = synth.catchment_case(n=n, DX=20.0, hours=72, lateral=True, storm_start_h=1.0)
        return case, 500, ("catchment %dx%d @20 m, erosion (Einstein, 9 fractions) + lateral3 + "
                           "slide_3, per-cell n; 60 mm/h storm from 60 min" % (n, n))
    if name == "flow8192":
        n = size or 8192
        case = synth.flow_case(n=n, DX=5.0, hours=2, grid_rain=True)
        return case, 1500, ("flow-only %dx%d @5 m, 30 mm/h on every cell (distributed "
                            "TOPMODEL runoff grid)" % (n, n))
    if name == "reach":
        case = synth.reach_case(imax=300, jmax=100, DX=10.0, hours=24)
        return case, 12000, "reach 300x100 @10 m, Wilcock, triangular hydrograph peaking at 6 h"
    raise SystemExit("unknown workload " + name)


def timed_from(desc, iteration, cycle):
    return "%s; timed from iteration %d (simulated minute %.1f)" % (desc, iteration, cycle)


# ---------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        time.sleep(0.2)
        rows = self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[3 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def spin_up(model, iterations, flags):
    """Runs the model for `iterations` iterations (or to the end of its run)."""
    t0 = time.perf_counter()
    left = iterations
    while left > 0:
        n = model.run(min(left, 2000), flags, records=False)
        left -= n
        s = model.scalars()
        log("spin-up: cycle %.1f min, iteration %d, %.1f s" % (s.cycle, s.counter,
                                                               time.perf_counter() - t0))
        if n == 0:
            break
    return model.scalars()


def spin_minutes(model, minutes, flags):
    """Runs the model in chunks of 500 iterations until the simulated clock
    passes `minutes` (the adjoint workload's runs)."""
    while True:
        n = model.run(500, flags, records=False)
        s = model.scalars()
        if s.cycle >= minutes or s.cycle / 60 >= model.p.maxcycle or n == 0:
            return s


def log(msg):
    print(msg, file=sys.stderr, flush=True)


# per-cell algorithmic bytes of flow_route: elevation, depth, qx, qy read and
# qx, qy written (48 B); + Manning's n (8 B) when spatially variable;
# + suspended load (Vsusptot read, qxs, qys written: 24 B) and the two
# vel_dir entries erosion consumes (16 B) when erosion is on.
#
# Per wet cell of one k_flow_route launch, from one ncu capture of the erosion
# catchment at 1400 x 1400 (the 2000 x 2000 state is beyond the capture size
# rule; the counts grow with the wet cells):
#   python bench.py --size 1400 --steps 20 --warmup 5 --profile-only 2 \
#       --profile-skip 20  under  ncu --clock-control none -k regex:k_flow_route
#       -c 1 --metrics dram__bytes_read.sum,dram__bytes_write.sum,
#       sm__inst_executed_pipe_fp64.sum,sm__pipe_fp64_cycles_active.sum
FLOW_CAPTURE = {"dram_bytes_per_wet_cell": 121.9, "fp64_warp_inst_per_wet_cell": 1.001,
                "source": "ncu capture of k_flow_route_q<1,5,1> (face-compacted, out-of-line "
                          "divisions), catchment 1400x1400, 500-iteration spin-up + 25 "
                          "iterations, 1,663,494 wet cells: 202.7 MB DRAM, 1.665 M FP64 warp "
                          "instructions; scaled by this launch's wet cells"}
FP64_LANES_PER_CLK_SM = 2  # this GPU's FP64 pipe: a warp instruction takes 16 cycles


def flow_bytes_per_cell(p):
    b = 48
    if p.spatially_var_mannings:
        b += 8
    if not p.hydro_only:
        b += 24 + 16
    return b


def aggregate_replicas(ms, done, dist, device="cpu"):
    """Replicas: the job's time is the slowest rank's, its work the sum of all
    ranks' steps (each rank runs its own full model).  Returns (max ms,
    total steps)."""
    if dist is None:
        return ms, done
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(done)], dtype=torch.float64, device=device)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), float(n.item())


# ---------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world, dist):
    import torch
    import hc
    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    t0 = time.perf_counter()
    case, spin_its, desc = make_workload(args.workload, args.size)
    if args.spinup >= 0:
        spin_its = int(args.spinup)
    log("workload generated in %.1f s" % (time.perf_counter() - t0))
    flags = case.flags
    model = hc.Model(case)
    spin_up(model, spin_its, flags)
    stream = torch.cuda.ExternalStream(model.stream())
    model.run(args.warmup, flags, records=False)
    log("warm-up done")
    if args.profile_only:
        if args.profile_skip:
            model.run(args.profile_skip, flags, records=False)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("profiled")
        prof = [model.profile_iteration(flags) for _ in range(args.profile_only)]
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        torch.cuda.nvtx.range_push("kernel")
        ms_flow, wet = model.bench_kernel("flow_route", 3)
        torch.cuda.nvtx.range_pop()
        phases = {k: float(np.mean([p_[k] for p_ in prof])) for k in prof[0]}
        return {"profile_only": True, "phases_ms": phases, "flow_route_ms": ms_flow,
                "wet_cells": wet}, model, case
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if clocks:
        clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = model.counters()[0]
    st0 = model.run_stats()
    sc0 = model.scalars()
    torch.cuda.nvtx.range_push("timed")
    e0.record(stream)
    done = model.run(args.steps, flags, records=False)
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = e0.elapsed_time(e1)
    launches = model.counters()[0] - l0
    sim_min = model.scalars().cycle - sc0.cycle
    st1 = model.run_stats()
    host_work = {k: {"count": st1[k][0] - st0[k][0], "host_ms": round(st1[k][1] - st0[k][1], 3)}
                 for k in st1 if k != "wet_cell_steps"}
    wet_steps = st1["wet_cell_steps"][0] - st0["wet_cell_steps"][0]
    clk = clocks.stop() if clocks else None
    ms, total_steps = aggregate_replicas(ms, done, dist, "cuda")
    cells = case.cells
    value = cells * total_steps / (ms / 1e3)
    out = {"ms": ms, "done": done, "value": value, "clocks": clk, "cells": cells,
           "spin_its": spin_its,
           "desc": timed_from(desc, int(sc0.counter) + 1, sc0.cycle),
           "launches": launches, "host_work": host_work, "sim_minutes": sim_min,
           "wet_cell_steps_per_s": wet_steps / (ms / 1e3) if world == 1 else None}
    if rank != 0 or args.timed_only:
        return out, model, case
    # the steps' periodic host work (lateral3 every 50 x erode_mult iterations,
    # a drainage recomputation when the baseflow threshold moves) falls
    # outside a short timed window: a longer window that holds at least one
    # of each, amortized per step
    if not case.params.hydro_only:
        out["amortized"] = amortized_window(model, case, flags, stream, args.amortize_max)
    # per-phase breakdown of a few iterations (phase by phase, no graph)
    nprof = int(os.environ.get("HC_PROFILE_ITERS", "60"))
    prof = [model.profile_iteration(flags) for _ in range(nprof)]
    out["phases_ms"] = {k: float(np.mean([p_[k] for p_ in prof])) for k in prof[0]}
    out["phases_ms"]["iterations_profiled"] = nprof
    # end-to-end through the public API: one hc_run call per step with the
    # step's record read back to host memory (the drop-in call pattern), on
    # a second model brought to the timed region's starting state (the runs
    # are deterministic), so that both numbers cover the same iterations
    e2e_steps = max(3, min(args.steps, 200))
    twin = hc.Model(case)
    spin_up(twin, spin_its, flags)
    # warm-up with records: the record buffer and the graphs that use it
    # exist before the timed calls
    twin.run(args.warmup, flags, records=True)
    torch.cuda.synchronize()
    _, h0, d0 = twin.counters()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        twin.run(1, flags, records=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    _, h1, d1 = twin.counters()
    twin.close()
    del twin
    # host wall clock: each call synchronises, so the host clock bounds the
    # device time and includes the per-call host work
    out["e2e"] = {"value": cells * e2e_steps / e2e_s, "unit": UNIT,
                  "h2d_bytes_per_step": (h1 - h0) // e2e_steps,
                  "d2h_bytes_per_step": (d1 - d0) // e2e_steps,
                  "steps": e2e_steps, "api": "hc_run(ctx, 1, flags, host_records) per step"}
    # the dominant kernel: its mean duration over the profiled iterations
    # (CUDA events around each launch on the library's stream, right after
    # the timed region), the launch processing the wet list
    ms_flow = out["phases_ms"]["flow_route"]
    _, wet = model.bench_kernel("flow_route", 1)
    peak, kind = measured_peak_hbm()
    per_cell = flow_bytes_per_cell(case.params)
    ach = wet * per_cell / (ms_flow / 1e3) / 1e9
    cap = FLOW_CAPTURE if not case.params.hydro_only else {}
    roof = {"bound": "hbm", "kernel": "k_flow_route", "achieved": ach, "peak": peak,
            "unit": "GB/s", "frac": ach / peak,
            "traffic": (cap["dram_bytes_per_wet_cell"] * wet
                        if cap.get("dram_bytes_per_wet_cell") else None),
            "traffic_source": cap.get("source"), "peak_kind": kind,
            "bytes_per_wet_cell": per_cell, "wet_cells": wet, "launch_ms": ms_flow}
    # the FP64 pipe, which bounds this kernel: its warp instructions per wet
    # cell (the capture) x 16 cycles each, against the pipe's cycles in the
    # launch at the SM clock sampled during the timed region
    if cap.get("fp64_warp_inst_per_wet_cell") and clk and clk.get("sm_mhz"):
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        need = cap["fp64_warp_inst_per_wet_cell"] * wet * (32 / FP64_LANES_PER_CLK_SM)
        have = sms * clk["sm_mhz"] * 1e6 * (ms_flow / 1e3)
        roof["fp64_pipe"] = {"frac": need / have, "warp_inst_per_wet_cell":
                             cap["fp64_warp_inst_per_wet_cell"], "sms": sms,
                             "sm_mhz": clk["sm_mhz"]}
    out["roofline"] = roof
    return out, model, case


def amortized_window(model, case, flags, stream, max_steps):
    """Runs on from the timed region in chunks of 50 iterations until the
    window holds a lateral3 call and a drainage recomputation (or max_steps);
    device time per step over the whole window, with the host work counted."""
    import torch
    st0 = model.run_stats()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    n = 0
    while n < max_steps:
        n += model.run(50, flags, records=False)
        st = model.run_stats()
        if (st["lateral"][0] > st0["lateral"][0] or not (flags & HC_RUN_LATERAL)) and \
                st["drainage"][0] > st0["drainage"][0]:
            break
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    st = model.run_stats()
    return {"steps": n, "ms_per_step": ms / max(1, n),
            "cell_steps_per_s": case.cells * n / (ms / 1e3),
            "lateral3_calls": st["lateral"][0] - st0["lateral"][0],
            "drainage_recomputations": st["drainage"][0] - st0["drainage"][0],
            "host_ms": round(sum(st[k][1] - st0[k][1] for k in st
                                 if k not in ("drainage_sweep", "wet_cell_steps")), 3),
            # wall time of each kind of host-driven work in the window (the
            # drainage kinds nest: sort, sweep and levels are parts of it)
            "host_work_ms": {k: round(st[k][1] - st0[k][1], 3) for k in st
                             if k != "wet_cell_steps" and st[k][1] - st0[k][1] > 0}}


def run_ensemble_bench(args, rank):
    """C5: independent catchments (synth.ensemble_member) advanced together by
    hc_run_ensemble, against the same members run one after the other with
    hc_run.  Both timed with the host clock between device-wide
    synchronisations (each member has its own stream)."""
    import torch
    import hc
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    n = args.members
    cases = [synth.ensemble_member(k, fill=False) for k in range(n)]
    log("%d members generated in %.1f s" % (n, time.perf_counter() - t0))
    models = [hc.Model(c) for c in cases]
    cells = sum(c.cells for c in cases)
    log("%d members on the device, %.1f M cells" % (n, cells / 1e6))
    warm = max(3, args.warmup)
    hc.run_ensemble(models, max(warm, args.spinup_iters), 0)
    torch.cuda.synchronize()
    k = args.steps
    # plain: one member after the other
    t0 = time.perf_counter()
    done_plain = [m.run(k, 0, records=False) for m in models]
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    # batched: all members in flight
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t0 = time.perf_counter()
    done = hc.run_ensemble(models, k, 0)
    torch.cuda.synchronize()
    t_ens = time.perf_counter() - t0
    clk = clocks.stop()
    # then per member, after the timed runs (each call returns after its
    # member's last iteration): the fixed cost per iteration against the
    # per-cell cost, least squares
    per = []
    for c_, m in zip(cases, models):
        t1 = time.perf_counter()
        m.run(k, 0, records=False)
        per.append((c_.cells, (time.perf_counter() - t1) * 1e3 / k))
    A = np.array([[1.0, c_] for c_, _ in per])
    fixed_ms, per_cell_ms = np.linalg.lstsq(A, np.array([t for _, t in per]), rcond=None)[0]
    log("plain per member: ms/iteration = %.4f + %.3e x cells" % (fixed_ms, per_cell_ms))
    steps_plain = sum(c.cells * d for c, d in zip(cases, done_plain))
    steps_ens = sum(c.cells * d for c, d in zip(cases, done))
    value = steps_ens / t_ens
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": k,
            "warmup": warm, "ms_per_step": t_ens * 1e3 / k, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generators, hail-caesar_gb300/synth.py)",
            "config": {"workload": "ensemble%d" % n, "members": n, "cells": cells,
                       "description": "%d independent catchments, sides 256-1536 @10 m, erosion "
                                      "+ slide_3, own dt each; %d iterations per member"
                                      % (n, k),
                       "parallelism": "one stream + graph per member",
                       "timing": "host clock between device synchronisations"},
            "clocks": clk, "plain_value": steps_plain / t_plain,
            "plain_ms_per_iteration_fit": {"fixed": fixed_ms, "per_mcell": per_cell_ms * 1e6},
            "batched_over_plain": (steps_ens / t_ens) / (steps_plain / t_plain)}


def run_adjoint_bench(args):
    """C4: gradient of the outlet-Q loss with respect to every cell's n and
    elevation and the rain table over --adj-iterations iterations (default
    4000), at most --adj-states model states kept (binomial checkpointing),
    against the same iterations run forward only."""
    import torch
    import hc
    torch.cuda.set_device(0)
    n_it = args.adj_iterations
    case = synth.adjoint_case(n=args.size or 1024)
    tcase = synth.adjoint_case(n=args.size or 1024, n_seed=99)
    spin = args.spinup if args.spinup >= 0 else 90.0

    def spun(c):
        m = hc.Model(c)
        spin_minutes(m, spin, 0)
        return m
    _, target = spun(tcase).adj_forward(n_it)
    mf = spun(case)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mf.run(n_it, 0, records=False)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    ma = spun(case)
    loss, gn, gr, info, ge = ma.adj_gradient(n_it, args.adj_states, target, elev=True)
    ratio = info["total_ms"] / (t_fwd * 1e3)
    cells = case.cells
    return {"metric": METRIC, "value": ratio, "unit": "adjoint/forward wall-time ratio",
            "n_gpus": 1, "steps": n_it, "warmup": 0, "ms_per_step": info["total_ms"] / n_it,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generators, hail-caesar_gb300/synth.py)",
            "config": {"workload": "adjoint%d" % (args.size or 1024), "cells": cells,
                       "description": "hydro-only %dx%d @10 m, 20 mm/h for 3 h; loss = MSE of "
                                      "outlet Q per simulated minute vs a run with another n "
                                      "field; gradient w.r.t. per-cell n, elevation and the rain "
                                      "table; binomial checkpointing" % (case.params.imax,
                                                                           case.params.jmax)},
            "forward_ms": t_fwd * 1e3, "forward_cell_steps_per_s": cells * n_it / t_fwd,
            "gradient_ms": {"forward_checkpointed": info["forward_ms"],
                            "reverse": info["reverse_ms"], "total": info["total_ms"],
                            "reverse_replays": info["replay_ms"],
                            "reverse_adjoint_iterations": info["adjoint_iterations_ms"]},
            "checkpointing": {"max_states": args.adj_states, "segment": info["segment"],
                              "snapshots": info["snapshots"],
                              "iterations_advanced_again": info["advanced"]},
            "loss": loss, "grad_n_norm": float(np.sqrt((gn ** 2).sum())),
            "grad_elev_norm": float(np.sqrt((ge ** 2).sum())),
            "grad_rain_norm": float(np.sqrt((gr ** 2).sum()))}


def cpu_sample(model, case, flags, budget_s=15.0):
    """The oracle port (OpenMP build) timed on the host from the GPU state."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    o = oracle.Oracle(case, omp=True)
    o.load_from(model)
    cores = os.cpu_count()
    n = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        if len(o.iterate(1, flags)) == 0:  # the run ended (maxcycle)
            break
        n += 1
    dt = time.perf_counter() - t0
    return {"value": case.cells * n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d steps from the GPU's timed state, %.1f s" % (n, dt)}


# ---------------------------------------------------------------- reference arm
def run_reference_ensemble(args, oracle):
    """The OpenMP port on a bounded sample of the ensemble: the first members,
    one after the other (the reference runs one catchment per process)."""
    n_sample = min(args.members, 4)
    steps = 0
    cells_steps = 0
    t_all = 0.0
    for k in range(n_sample):
        case = synth.ensemble_member(k, fill=False)
        o = oracle.Oracle(case, omp=True)
        o.iterate(max(3, args.warmup), 0)
        m = max(1, min(args.steps, 40))
        t0 = time.perf_counter()
        o.iterate(m, 0)
        t_all += time.perf_counter() - t0
        cells_steps += case.cells * m
        steps += m
    v = cells_steps / t_all
    cores = os.cpu_count()
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_all * 1e3 / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "ensemble%d" % args.members,
                                            "members": args.members},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "members 0-%d, %d iterations in all, OpenMP port"
                                       % (n_sample - 1, steps)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference(args):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    if args.workload == "ensemble":
        return run_reference_ensemble(args, oracle)
    if args.workload == "adjoint":
        return {"impl": "reference", "unavailable": "the reference has no adjoint of its "
                "iteration; nothing to time on the CPU for this workload"}
    case, spin_its, desc = make_workload(args.workload, args.size)
    if args.spinup >= 0:
        spin_its = int(args.spinup)
    flags = case.flags
    o = oracle.Oracle(case, omp=True)
    # the same iterations as the GPU arm: spin-up, warm-up, then the timed
    # steps of the same deterministic run
    o.iterate(spin_its, flags)
    o.iterate(args.warmup, flags)
    it0, cyc0 = int(o.scalar("counter")), o.scalar("cycle")
    t0 = time.perf_counter()
    o.iterate(args.steps, flags)
    dt = time.perf_counter() - t0
    v = case.cells * args.steps / dt
    cores = os.cpu_count()
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": DATA, "config": workload_config(args, case, timed_from(desc, it0 + 1, cyc0),
                                                    spin_its),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d steps after %d spin-up + %d warm-up iterations, OpenMP "
                                       "port (-O3) on %d threads" % (args.steps, spin_its,
                                                                     args.warmup, cores)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="catchment2000",
                    choices=["catchment2000", "flow8192", "reach", "ensemble", "adjoint"])
    ap.add_argument("--members", type=int, default=96, help="ensemble members")
    ap.add_argument("--adj-iterations", type=int, default=4000,
                    help="adjoint: iterations of the differentiated run")
    ap.add_argument("--adj-states", type=int, default=220,
                    help="adjoint: model states kept at once (binomial checkpointing)")
    ap.add_argument("--spinup-iters", type=int, default=300,
                    help="ensemble: iterations each member runs before timing")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--size", type=int, default=0,
                    help="override the grid side (smaller runs for profiling)")
    ap.add_argument("--spinup", type=float, default=-1,
                    help="override the spin-up: iterations (simulated minutes for the "
                         "adjoint workload)")
    ap.add_argument("--amortize-max", type=int, default=1000,
                    help="longest window of the amortized per-step figure")
    ap.add_argument("--timed-only", action="store_true",
                    help="only the timed steps (no e2e, profile, kernel timing or CPU leg); "
                         "for runs under a profiler")
    ap.add_argument("--profile-skip", type=int, default=0, metavar="S",
                    help="with --profile-only: run S iterations first (e.g. --steps, to "
                         "profile the state at the end of the timed region)")
    ap.add_argument("--profile-only", type=int, default=0, metavar="N",
                    help="after the warm-up, run N iterations launch by launch (no graph) "
                         "inside the NVTX range 'profiled', then the dominant kernel alone "
                         "inside 'kernel'; for profilers that do not see into graphs")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if args.workload == "ensemble":
        if rank == 0:
            print(json.dumps(run_ensemble_bench(args, rank)))
        return
    if args.workload == "adjoint":
        if rank == 0:
            print(json.dumps(run_adjoint_bench(args)))
        return
    dist = None
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
        dist = tdist
    out, model, case = run_gpu(args, rank, world, dist)
    if rank == 0 and args.profile_only:
        print(json.dumps(out))
    elif rank == 0 and args.timed_only:
        print(json.dumps({"timed_only": True, "ms_per_step": out["ms"] / max(1, out["done"]),
                          "value": out["value"], "launches": out["launches"]}))
    elif rank == 0:
        line = {
            "metric": METRIC, "value": out["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["ms"] / out["done"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": DATA, "config": workload_config(args, case, out["desc"], out["spin_its"]),
            "clocks": out["clocks"], "e2e": out["e2e"], "roofline": out["roofline"],
            "gpu_launches": out["launches"], "phases_ms": out["phases_ms"],
            "wet_cell_steps_per_s": out["wet_cell_steps_per_s"],
            "amortized": out.get("amortized"),
            "host_work": out["host_work"], "simulated_minutes_timed": out["sim_minutes"],
        }
        if world == 1:
            line["cpu_baseline"] = cpu_sample(model, case, case.flags, args.cpu_budget)
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
