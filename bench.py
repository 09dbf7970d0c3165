"""Benchmark: cell-steps/s of HAIL-CAESAR's per-timestep raster path on GB300.

One step = one iteration of the reference's main loop (src/main.cpp:139-204):
inputs, flow_route, depth_update, the Courant dt, scan_area, erosion/deposition
with grain sorting, lateral3, water_flux_out and slide_3, on one batch of
synthetic input already resident in HBM.

Workloads (seeded synthetic inputs with the benchmark configurations' shapes):
  catchment2000  (default) catchment mode, 2000 x 2000 cells at 20 m, fractal
                 DEM with 300 m relief pit-filled to one outlet edge,
                 gamma rain + 60 mm/h storm, per-cell Manning's n, Einstein
                 transport, lateral3 and slide_3 on; the storm starts at
                 1 h and the timed steps begin 30 min into it
  flow8192       flow-only 8192 x 8192 at 5 m, 30 mm/h rain, erosion off
  reach          reach mode 300 x 100 at 10 m, Wilcock-Crowe

--impl gb300 (default) times libhc_gpu; --impl reference times the CPU
implementation of the path (the oracle port, OpenMP over the reference's own
column loops) on the host cores, from the same spun-up state definition.

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


def make_workload(name, size=0):
    """(case, spin-up simulated minutes, description)."""
    if name == "catchment2000":
        case = synth.catchment_case(n=size or 2000, DX=20.0, hours=72, lateral=True,
                                    storm_start_h=1.0)
        return case, 90.0, ("catchment 2000x2000 @20 m, erosion + lateral3 + slide_3, timed 30 min "
                            "into the 60 mm/h storm (storm from 1 h, spin-up to 1.5 h)")
    if name == "flow8192":
        case = synth.flow_case(n=size or 8192, DX=5.0, hours=2)
        return case, 75.0, "flow-only 8192x8192 @5 m, 30 mm/h, after 75 min"
    if name == "reach":
        case = synth.reach_case(imax=300, jmax=100, DX=10.0, hours=24)
        return case, 6 * 60.0, "reach 300x100 @10 m, Wilcock, after 6 h (hydrograph peak)"
    raise SystemExit("unknown workload " + name)


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


def spin_up(model, minutes, flags):
    """Runs the model until the simulated clock passes `minutes`."""
    t0 = time.perf_counter()
    while True:
        n = model.run(500, flags, records=False)
        s = model.scalars()
        log("spin-up: cycle %.1f min, iteration %d, %.1f s" % (s.cycle, s.counter,
                                                               time.perf_counter() - t0))
        if s.cycle >= minutes or s.cycle / 60 >= model.p.maxcycle or n == 0:
            return s


def log(msg):
    print(msg, file=sys.stderr, flush=True)


# per-cell algorithmic bytes of flow_route: elevation, depth, qx, qy read and
# qx, qy written (48 B); + Manning's n (8 B) when spatially variable;
# + suspended load (Vsusptot read, qxs, qys written: 24 B) and the two
# vel_dir entries erosion consumes (16 B) when erosion is on.
TRAFFIC_SED_FLOW = 121.6  # B per wet cell, profiles/k_flow_route_catchment1400.md


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
    case, spin_min, desc = make_workload(args.workload, args.size)
    if args.spinup >= 0:
        spin_min = args.spinup
    log("workload generated in %.1f s" % (time.perf_counter() - t0))
    flags = case.flags
    model = hc.Model(case)
    spin_up(model, spin_min, flags)
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
    cyc0 = model.scalars().cycle
    torch.cuda.nvtx.range_push("timed")
    e0.record(stream)
    done = model.run(args.steps, flags, records=False)
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = e0.elapsed_time(e1)
    launches = model.counters()[0] - l0
    sim_min = model.scalars().cycle - cyc0
    st1 = model.run_stats()
    host_work = {k: {"count": st1[k][0] - st0[k][0], "host_ms": round(st1[k][1] - st0[k][1], 3)}
                 for k in st1}
    clk = clocks.stop() if clocks else None
    ms, total_steps = aggregate_replicas(ms, done, dist, "cuda")
    cells = case.cells
    value = cells * total_steps / (ms / 1e3)
    out = {"ms": ms, "done": done, "value": value, "clocks": clk, "cells": cells, "desc": desc,
           "launches": launches, "host_work": host_work, "sim_minutes": sim_min}
    if rank != 0 or args.timed_only:
        return out, model, case
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
    spin_up(twin, spin_min, flags)
    twin.run(args.warmup, flags, records=False)
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
    # dominant kernel, timed alone with events on the library's stream
    reps = 20
    ms_flow, wet = model.bench_kernel("flow_route", reps)
    peak, kind = measured_peak_hbm()
    per_cell = flow_bytes_per_cell(case.params)
    ach = wet * per_cell / (ms_flow / 1e3) / 1e9
    # DRAM bytes per wet cell of one k_flow_route launch, from the ncu
    # capture summarised in profiles/ (a smaller case of the same generator),
    # scaled to this launch by its wet cells
    traffic_per_cell = None if case.params.hydro_only else TRAFFIC_SED_FLOW
    out["roofline"] = {"bound": "hbm", "kernel": "k_flow_route", "achieved": ach, "peak": peak,
                       "unit": "GB/s", "frac": ach / peak,
                       "traffic": None if traffic_per_cell is None else traffic_per_cell * wet,
                       "peak_kind": kind, "bytes_per_wet_cell": per_cell, "wet_cells": wet,
                       "launch_ms": ms_flow,
                       "limiter": "FP64 pipe (ncu: 67 % of its issue slots, ALU 42 %, DRAM 9 %)"}
    return out, model, case


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
            "batched_over_plain": (steps_ens / t_ens) / (steps_plain / t_plain)}


def run_adjoint_bench(args):
    """C4: gradient of the outlet-Q loss with respect to every cell's n and
    the rain table over `--steps` iterations (default 4000), checkpoints
    every 200, against the same iterations run forward only."""
    import torch
    import hc
    torch.cuda.set_device(0)
    n_it = args.adj_iterations
    case = synth.adjoint_case(n=args.size or 1024)
    tcase = synth.adjoint_case(n=args.size or 1024, n_seed=99)
    spin = args.spinup if args.spinup >= 0 else 90.0

    def spun(c):
        m = hc.Model(c)
        spin_up(m, spin, 0)
        return m
    _, target = spun(tcase).adj_forward(n_it)
    mf = spun(case)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mf.run(n_it, 0, records=False)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    ma = spun(case)
    loss, gn, gr, ms = ma.adj_gradient(n_it, 200, target)
    ratio = ms[2] / (t_fwd * 1e3)
    cells = case.cells
    return {"metric": METRIC, "value": ratio, "unit": "adjoint/forward wall-time ratio",
            "n_gpus": 1, "steps": n_it, "warmup": 0, "ms_per_step": ms[2] / n_it,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generators, hail-caesar_gb300/synth.py)",
            "config": {"workload": "adjoint%d" % (args.size or 1024), "cells": cells,
                       "description": "hydro-only %dx%d @10 m, 20 mm/h for 3 h; loss = MSE of "
                                      "outlet Q per simulated minute vs a run with another n "
                                      "field; gradient w.r.t. per-cell n and the rain table; "
                                      "checkpoints every 200 iterations" % (case.params.imax,
                                                                           case.params.jmax)},
            "forward_ms": t_fwd * 1e3, "forward_cell_steps_per_s": cells * n_it / t_fwd,
            "gradient_ms": {"forward_checkpointed": ms[0], "reverse": ms[1], "total": ms[2]},
            "loss": loss, "grad_n_norm": float(np.sqrt((gn ** 2).sum())),
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
        o.iterate(1, flags)
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
    case, spin_min, desc = make_workload(args.workload, args.size)
    flags = case.flags
    o = oracle.Oracle(case, omp=True)
    while True:
        o.iterate(2000, flags)
        if o.scalar("cycle") >= spin_min:
            break
    o.iterate(args.warmup, flags)
    t0 = time.perf_counter()
    o.iterate(args.steps, flags)
    dt = time.perf_counter() - t0
    v = case.cells * args.steps / dt
    cores = os.cpu_count()
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": args.workload, "description": desc,
                                            "cells": case.cells},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d steps after spin-up, OpenMP port" % args.steps},
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
    ap.add_argument("--spinup-iters", type=int, default=300,
                    help="ensemble: iterations each member runs before timing")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--size", type=int, default=0,
                    help="override the grid side (smaller runs for profiling)")
    ap.add_argument("--spinup", type=float, default=-1,
                    help="override the spin-up, simulated minutes")
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
            "data": "synthetic (seeded generators, hail-caesar_gb300/synth.py)",
            "config": {"workload": args.workload, "description": out["desc"],
                       "cells": out["cells"], "parallelism": "replicas x%d" % world,
                       "l2": "inputs larger than L2 (model state several GB)"},
            "clocks": out["clocks"], "e2e": out["e2e"], "roofline": out["roofline"],
            "gpu_launches": out["launches"], "phases_ms": out["phases_ms"],
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
