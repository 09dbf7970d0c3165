/* libhc_gpu: GB300 (sm_103a) implementation of HAIL-CAESAR's per-timestep
 * raster path, behind a plain C ABI.
 *
 * The reference has no plugin API: its hot path is the set of argument-free
 * member functions of LSDCatchmentModel that src/main.cpp:139-204 calls once
 * per iteration, all communicating through private TNT arrays.  Each entry
 * point below names the member function it replaces (file:line in the
 * reference, src/catchmentmodel/LSDCatchmentModel.cpp unless stated).  The
 * model state lives in device memory owned by an hc_ctx; hc_upload/
 * hc_download move whole fields in the reference's own (TNT, padded,
 * row-major) layout, so the host side keeps its arrays unchanged.
 *
 * Every call returns an hc_status; the library never exits the process.
 * One host thread per context; all work is ordered on the context's stream.
 */
#ifndef HC_GPU_H
#define HC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HC_G_MAX 10      /* LSDCatchmentModel.hpp:444 (grain fractions + 1) */
#define HC_NSTRATA 10    /* strata layers, LSDCatchmentModel.cpp:1759 */
#define HC_MAX_RF 16     /* largest rfnum (hydroindex rain zones) supported */
#define HC_MAX_POINTS 3  /* reach input points, LSDCatchmentModel.cpp:1742-1800 */

typedef enum hc_status {
  HC_OK = 0,
  HC_ERR_ARG = 1,        /* bad argument: null pointer, size, unknown field */
  HC_ERR_CUDA = 2,       /* a CUDA call failed; see hc_last_error */
  HC_ERR_NONFINITE = 3,  /* a NaN/Inf water depth was detected */
  HC_ERR_TIMEOUT = 4,    /* a device wait gave up (bounded spin) */
  HC_ERR_NOMEM = 5,      /* device allocation failed or exceeds the cap */
  HC_ERR_STATE = 6,      /* call out of order (e.g. run before prepare) */
  HC_ERR_UNSUPPORTED = 7 /* option outside what the library implements */
} hc_status;

/* Every scalar the path reads.  Defaults (hc_params_default) are the
 * reference's member initialisers, LSDCatchmentModel.hpp:437-568, and the
 * driver constants of main.cpp:127-132. */
typedef struct hc_params {
  int32_t imax, jmax;     /* rows (DEM nrows) and columns (DEM ncols) */
  double DX;              /* cell size, m */
  /* flow routing */
  double courant_number;
  double froude_limit;
  double mannings;
  double hflow_threshold;
  double edgeslope;
  double water_depth_erosion_threshold; /* fixed 0.01 in the reference */
  double in_out_difference_allowed;
  int32_t max_time_step;  /* s */
  int32_t spatially_var_mannings;
  double ERODEFACTOR;     /* key erosion_limit */
  int32_t maxcycle;       /* hours (key max_run_duration) */
  /* rainfall / TOPMODEL (uniform or hydroindex-zoned rain) */
  double rain_data_time_step; /* minutes */
  int32_t rfnum;
  double M;
  double rain_factor;
  double baseflow;
  double MIN_Q, MIN_Q_MAXVAL;
  /* reach inputs */
  int32_t reach_mode;
  int32_t number_of_points;
  int32_t inpoints[HC_MAX_POINTS][2];
  int32_t reach_input_data_timestep; /* minutes */
  int32_t div_inputs;
  /* sediment */
  int32_t hydro_only;
  int32_t wilcock, einstein;
  double active;
  double max_vel;
  double Csuspmax;
  double bedrock_erosion_threshold;
  double bedrock_erosion_rate;
  double vegTauCrit;
  double veg_lat_restriction;
  double lateral_constant;
  double chann_lateral_erosion;
  double failureangle;
  double CREEP_RATE;
  double d[HC_G_MAX];          /* d[1..9] grain sizes, m */
  double dprop[HC_G_MAX + 1];  /* dprop[0..10] */
  double fallVelocity[HC_G_MAX + 1];
  int32_t isSuspended[HC_G_MAX + 1];
  int32_t vegetation_on;
  /* lateral3 */
  double edge_smoothing_passes;
  double downstream_shift;
  double lateral_cross_channel_smoothing;
  /* driver intervals, main.cpp:127-132 */
  int32_t scan_area_interval_iter;
  int32_t in_channel_landslide_iter_interval;
  int32_t creep_time_interval;
  int32_t global_landsliding_interval;
  double creep_coeff;
  int32_t LIMIT;
  /* distributed TOPMODEL rainfall-runoff: every cell of the grid takes its
   * own runoff (catchment_water_input_and_hydrology(flow_timestep, runoff)
   * :3544-3607, runoffGrid::calculate_runoff LSDRainfallRunoff.cpp:175-241,
   * key spatially_complex_rainfall_on :1355); 0: zoned TOPMODEL through the
   * catchment input points */
  int32_t spatially_complex_rainfall;
} hc_params;

/* Scalar state of the model object (members of LSDCatchmentModel that the
 * per-step path reads or writes).  Kept on the device during a run. */
typedef struct hc_scalars {
  double cycle, previous, time_step, maxdepth;
  double waterinput, waterOut, input_output_difference, temptot;
  double counter, erode_call, erode_mult, lateralcounter;
  double time_1, baseflow, grain_array_tot;
  double sediQ, globalsediq, tempbmax;
  double creep_time, creep_time2;
  double sum_grain[HC_G_MAX + 1];
  double j[HC_MAX_RF + 1], jo[HC_MAX_RF + 1], j_mean[HC_MAX_RF + 1];
  double old_j_mean[HC_MAX_RF + 1], new_j_mean[HC_MAX_RF + 1];
  double nActualGridCells[HC_MAX_RF + 1];
  double catchment_input_counter[HC_MAX_RF + 1];
  double totalinputpoints;
  double flow_timestep;   /* flow dt of the current iteration */
  double stop_flag;       /* nonzero: host-side work needed before resuming */
} hc_scalars;

/* Per-iteration record of hc_run.  The first ten fields are those of
 * oracle/ref_harness (the reference's own members after the iteration).  The
 * last four are the water ledger of the iteration, which the reference does
 * not keep (its waterinput / waterOut are rates for the time-step control):
 *   vol_in   water the inputs added to the grid (reach points, catchment
 *            input points, distributed runoff), m^3;
 *   vol_out  water water_flux_out took off the edges plus water depth_update
 *            zeroed at no-data cells, m^3;
 *   vol_mask water that crossed a face between a cell of the wet list and
 *            one outside it, m^3 (signed: + appeared, - vanished).  The
 *            reference updates only listed cells (down_scan, rebuilt every
 *            scan_area_interval_iter iterations), so such a face changes one
 *            side's depth only; this is the one place its scheme does not
 *            conserve water;
 *   volume   sum of water depth x DX^2 over the grid (rows 1..imax, columns
 *            1..jmax) right after depth_update, m^3, on iterations that run
 *            scan_area (the full-grid pass that measures it); NaN on others. */
typedef struct hc_step_record {
  double counter, cycle, time_step, maxdepth, waterOut, waterinput,
      erode_mult, sediQ, globalsediq, baseflow;
  double vol_in, vol_out, vol_mask, volume;
} hc_step_record;

/* Fields that hc_upload / hc_download move, in the reference's layouts. */
typedef enum hc_field {
  HC_F_ELEV = 0,         /* double (imax+2)(jmax+2) */
  HC_F_WATER_DEPTH,      /* double (imax+2)(jmax+2) */
  HC_F_QX, HC_F_QY, HC_F_QXS, HC_F_QYS, /* double (imax+2)(jmax+2) */
  HC_F_VSUSPTOT,         /* double (imax+2)(jmax+2) */
  HC_F_VEL, HC_F_TAU,    /* double (imax+2)(jmax+2) */
  HC_F_BEDROCK,          /* double (imax+2)(jmax+2) */
  HC_F_MANNINGS,         /* double (imax+2)(jmax+2) spat_var_mannings */
  HC_F_AREA,             /* double (imax+2)(jmax+2) drainage area */
  HC_F_SS,               /* double (imax+2)(jmax+2) */
  HC_F_VEL_DIR,          /* double (imax+2)(jmax+2)*9 */
  HC_F_SR, HC_F_SL, HC_F_SU, HC_F_SD, /* double (imax+2)(jmax+2)*10 */
  HC_F_INDEX,            /* int32 (imax+2)(jmax+2), -9999 = no grain record */
  HC_F_GRAIN,            /* double (imax+2)(jmax+2)/LIMIT * 11, by index */
  HC_F_STRATA,           /* double (imax+2)(jmax+2)/LIMIT * 10 * 11 */
  HC_F_DOWN_SCAN,        /* int32 (jmax+2)(imax+2) wet-row lists */
  HC_F_EDGE,             /* double (imax+1)(jmax+1) */
  HC_F_VEG,              /* double (imax+1)(jmax+1)*4 */
  HC_F_RFAREA,           /* int32 (imax+2)(jmax+2) */
  HC_F_INPUTPOINTS,      /* uint8 (imax+2)(jmax+2) reach input mask */
  HC_F_COUNT
} hc_field;

typedef struct hc_ctx hc_ctx;

/* Run flags (hc_run and the oracle's hco_iterate). */
#define HC_RUN_LATERAL 1  /* call lateral3 after erosion (main.cpp:178) */
#define HC_RUN_NOHILL 2   /* skip creep and global landsliding */

/* Fills p with the reference defaults for an imax x jmax grid of cell DX. */
void hc_params_default(hc_params* p, int32_t imax, int32_t jmax, double DX);

/* Element count and element size of a field for the given parameters. */
int64_t hc_field_count(const hc_params* p, hc_field f);
int32_t hc_field_elsize(hc_field f);

/* Allocates the device mirror of the model state and zeroes it like
 * initialise_arrays + zero_values (:1617-1843, :2891-2982).  max_bytes caps
 * the device allocation (0 = no cap). */
hc_status hc_create(const hc_params* p, size_t max_bytes, hc_ctx** out);
hc_status hc_destroy(hc_ctx* ctx);
const char* hc_last_error(const hc_ctx* ctx);

/* Copies a whole field host->device / device->host (synchronous w.r.t.
 * the host buffer).  nbytes must equal count*elsize. */
hc_status hc_upload(hc_ctx* ctx, hc_field f, const void* host, size_t nbytes);
hc_status hc_download(hc_ctx* ctx, hc_field f, void* host, size_t nbytes);

/* Rain table (rows x cols float, mm/h, read_rainfalldata :532-556) and reach
 * table of input point p (rows x cols float, read_reachfile :558-606). */
hc_status hc_set_rain(hc_ctx* ctx, const float* rain, int32_t rows, int32_t cols);
hc_status hc_set_reach(hc_ctx* ctx, int32_t point, const float* data,
                       int32_t rows, int32_t cols);

hc_status hc_get_scalars(hc_ctx* ctx, hc_scalars* s);
hc_status hc_set_scalars(hc_ctx* ctx, const hc_scalars* s);

/* Set-up that main.cpp:102-122 does once: count_catchment_gridcells (:2813),
 * set_time_counters (:1862), initialise_rainfall_runoff (:2041),
 * initialise_drainage_area (:2055).  Call after the fields are uploaded. */
hc_status hc_prepare(hc_ctx* ctx);

/* ---- member-level entry points (one reference member each) ---- */
/* set_maximum_timestep :1890-1910 (with set_inputoutput_diff :1879) */
hc_status hc_set_maximum_timestep(hc_ctx* ctx);
/* flow_route :3063-3247, dt = get_flow_timestep :1913-1923 */
hc_status hc_flow_route(hc_ctx* ctx);
/* depth_update :3259-3299; maxdepth lands in the scalars */
hc_status hc_depth_update(hc_ctx* ctx);

/* depth_update :3259-3299 on caller-owned device buffers, allocating nothing.
 * No counterpart in the reference (its member works on the object's own
 * arrays).  For callers that cannot allocate: a program that mirrors the TNT
 * arrays in device memory of its own under a fixed budget (cudaMalloc would
 * fail there), or that shares the GPU with other streams (cudaFree waits for
 * the whole device).  Buffers are device pointers in the reference's layout:
 * fields (imax+2)*(jmax+2) doubles, down_scan (jmax+2)*(imax+2) int32 lists
 * of distinct rows as scan_area writes them.  Vsusptot may be null (no
 * suspended fraction); if given, qxs and qys are needed.  *maxdepth (device)
 * receives the reference's maxdepth.  flow_timestep is get_flow_timestep's
 * value.  The call is asynchronous on `stream` (a cudaStream_t, 0 for the
 * legacy stream) on the current device.  Working memory is one fixed array
 * of the library (128 KiB per device), so jmax is limited to
 * HC_DEPTH_NOALLOC_MAX_COLS; larger grids get HC_ERR_ARG.  The first call on
 * each device looks up that array's address, so make it before any stream
 * capture.  All calls on a device share the array: calls that overlap in
 * time (other streams, other threads) race; order them on one stream.  err
 * (optional, err_len bytes) receives a one-line reason for a failure. */
#define HC_DEPTH_NOALLOC_MAX_COLS 16383
hc_status hc_depth_update_noalloc(int32_t imax, int32_t jmax, double DX, double flow_timestep,
                                  const int32_t* down_scan, const double* elev,
                                  const double* qx, const double* qy, const double* qxs,
                                  const double* qys, double* water_depth, double* Vsusptot,
                                  double* maxdepth, void* stream, char* err, size_t err_len);
/* The order drainage_area_D8 sweeps the cells in (:2091-2180): the
 * permutation std::sort (GCC's introsort) gives (key, value) pairs compared
 * by value only, equal values in std::sort's own order.  perm[k] receives the
 * index of the value at sorted position k; hc_run calls the same sort with
 * the reference's padded pair vector.  Runs on the current device;
 * *on_device (optional) is 0 when the host's exact sort ran instead (an
 * input that exhausts the introsort's depth budget, or a NaN). */
hc_status hc_drainage_sort(const double* values, uint64_t n, uint32_t* perm, int32_t* on_device);
/* scan_area :3821-3849 */
hc_status hc_scan_area(hc_ctx* ctx);
/* water_flux_out :3005-3047 */
hc_status hc_water_flux_out(hc_ctx* ctx);
/* erode(mult) :4211-4845; returns tempbmax */
hc_status hc_erode(hc_ctx* ctx, double mult, double* tempbmax);
/* lateral_channel_erode :4850-5291 */
hc_status hc_lateral_channel_erode(hc_ctx* ctx);
/* in_channel_landsliding :5429-5527 */
hc_status hc_in_channel_landsliding(hc_ctx* ctx);
/* global_landsliding :5529-5654 (daily in main.cpp's loop, call_global_landsliding
 * :1986-1996); *sweeps (optional) receives the number of sweeps made */
hc_status hc_global_landsliding(hc_ctx* ctx, int32_t* sweeps);
/* creep(time) :5293-5427 (every creep_time_interval minutes, slope_creep
 * :1976-1984, with time = creep_coeff) */
hc_status hc_creep(hc_ctx* ctx, double time);

/* ---- whole iterations ----
 * Runs up to n iterations of main.cpp:139-204 on the device (the same
 * member sequence as above, with the scalar logic of set_loop_cycle,
 * set_inputoutput_diff, set_maximum_timestep, increment_counters,
 * reach_water_and_sediment_input, catchment_waterinputs, call_erosion,
 * call_lateral and call_channel_landsliding kept on the device), stopping
 * early when cycle/60 >= maxcycle.  rec (may be NULL) receives one record per
 * iteration.  *done = iterations run. */
hc_status hc_run(hc_ctx* ctx, int64_t n, int32_t flags, hc_step_record* rec,
                 int64_t* done);

/* Water-mass ledger (no counterpart in the reference; its only ledger is the
 * pair of rates waterinput :3435/:3460 and waterOut :3046 that
 * set_maximum_timestep :1905 compares).  Volumes in m^3, accumulated by every
 * iteration (and member call) since hc_prepare or hc_mass_reset:
 *   volume - (volume0 + inflow - outflow - lost + mask_edge)
 * is what is left unexplained: rounding only, since every other face flux
 * leaves one cell and enters its neighbour.  hc_mass_balance measures
 * `volume` now, with a deterministic device reduction over rows 1..imax,
 * columns 1..jmax. */
typedef struct hc_mass {
  double volume0;    /* water on the grid when the ledger started */
  double volume;     /* water on the grid now */
  double inflow;     /* added by the inputs (reach, catchment points, runoff) */
  double outflow;    /* taken off the edges by water_flux_out */
  double lost;       /* zeroed by depth_update at no-data cells */
  double mask_edge;  /* net water that crossed faces at the wet list's border
                        (see hc_step_record::vol_mask) */
} hc_mass;
hc_status hc_mass_balance(hc_ctx* ctx, hc_mass* m);
/* Starts the ledger again from the water on the grid now. */
hc_status hc_mass_reset(hc_ctx* ctx);

/* Raster output while the run goes on (no counterpart in the reference,
 * which writes between iterations): hc_snapshot_begin copies a field with a
 * plain layout (elev, water_depth, qx, qy, Vsusptot, Vel, Tau, bedrock,
 * Manning's n, area, ss, edge) in stream order and moves the copy to
 * `host_pinned` (page-locked memory of nbytes) on a side stream, so hc_run
 * may be called again at once; hc_snapshot_end waits for the copy and frees
 * the snapshot.  The host buffer must stay valid until then. */
typedef struct hc_snapshot hc_snapshot;
hc_status hc_snapshot_begin(hc_ctx* ctx, hc_field f, void* host_pinned, size_t nbytes,
                            hc_snapshot** out);
hc_status hc_snapshot_end(hc_snapshot* snap);

/* Ensemble (no counterpart in the reference, which runs one catchment per
 * process): runs up to n iterations of each of m independent contexts at
 * once, each on its own stream with its own CUDA graph, adaptive dt and
 * host-side steps; done[k] receives member k's iteration count.  Members may
 * differ in size and parameters.  The members are serviced by up to 32 host
 * threads (member k by thread k mod T), so one member's host-side step
 * holds up only the members of its thread; a member must not be used by
 * another thread during the call. */
hc_status hc_run_ensemble(hc_ctx** ctxs, int32_t m, int64_t n, int32_t flags, int64_t* done);

/* ---- adjoint of the hydraulic iteration (no counterpart in the reference)
 * Hydro-only runs.  The outlet discharge Q (water_flux_out's sum) is
 * sampled at the first iteration of every simulated minute.
 *
 * hc_adj_forward runs n iterations like hc_run and returns the Q samples.
 * rec_out (optional, n*HC_ADJ_RECORD doubles) receives each iteration's
 * time steps; passing such a record as `fixed` imposes those time steps
 * instead of the adaptive ones (finite-difference runs of a perturbed model).
 *
 * hc_adj_gradient runs n iterations from the current state, evaluates
 * loss = mean over the samples of (Q - q_target)^2 and its gradient with
 * respect to every cell's Manning's n (grad_n), every cell's elevation
 * (grad_elev; both (imax+2)(jmax+2) doubles) and every entry of the rain
 * table (grad_rain: rows x cols as given to hc_set_rain).  Time steps, wet
 * mask and input points are held at the run's values (they are piecewise
 * constant in the parameters).  Memory: at most max_states model states
 * (h, qx, qy, wet mask: 25 bytes a cell each) are kept at once, as
 * binomial checkpoints (Griewank's revolve) of segments of K iterations plus
 * the K iteration states of the segment being reversed, or of two segments
 * when the cap allows it without more recomputation: then one segment is
 * replayed while the adjoint iterations of the next run on a second stream.
 * K is the one with the least recomputation.  The model is left at the end
 * of the n iterations.  ms (optional, 8 doubles): forward ms, reverse ms,
 * total ms, K, snapshots, iterations run again beyond the forward run and
 * the segments' replays, then the reverse's parts, which overlap: host ms
 * replaying the segments (keeping their states), device ms of the adjoint
 * iterations. */
#define HC_ADJ_RECORD 22
hc_status hc_adj_forward(hc_ctx* ctx, int64_t n, const double* fixed, double* rec_out,
                         double* q_samples, int64_t q_cap, int64_t* n_samples);
hc_status hc_adj_gradient(hc_ctx* ctx, int64_t n, int32_t max_states, const double* q_target,
                          int64_t n_target, double* loss, double* grad_n, double* grad_rain,
                          double* grad_elev, double* ms);

/* What hc_run spent on the host (no counterpart in the reference): for
 * each kind below, how many times it ran and its host wall time in ms,
 * accumulated since hc_create.  Pauses leave the rest of a graph chunk as
 * no-op iterations; HC_STAT_IDLE_ITERS counts those. */
enum {
  HC_STAT_CHUNKS = 0,      /* graph launches */
  HC_STAT_ERODE_RETRY,     /* erosion retries past the captured passes */
  HC_STAT_LATERAL,         /* lateral3 runs (host-driven convergence loop) */
  HC_STAT_CREEP,           /* slope creep */
  HC_STAT_GLOBAL_SLIDE,    /* global landsliding */
  HC_STAT_DRAINAGE,        /* drainage area + input points (baseflow change) */
  HC_STAT_DRAINAGE_SORT,   /* of those, sorts of the elevations (equal elevations that matter) */
  HC_STAT_DRAINAGE_SWEEP,  /* device accumulation (ms: device time) */
  HC_STAT_DRAINAGE_LEVELS, /* frontiers the accumulations went through (count) */
  HC_STAT_IDLE_ITERS,      /* captured iterations skipped after a pause */
  HC_STAT_DRAINAGE_HOST_SORT, /* of the sorts, those the host finished (see hc_drainage_sort) */
  HC_STAT_WET_CELL_STEPS,  /* count: wet-list cells summed over the iterations run (the
                              cells the reference's down_scan loops visit) */
  HC_STAT_COUNT
};
hc_status hc_get_run_stats(hc_ctx* ctx, int64_t* counts, double* host_ms, int32_t n);

/* Test hook of the bounded device waits (no counterpart in the reference).
 * The drainage recomputation (drainage_area_D8 :2091-2271) runs as one
 * cooperative kernel whose blocks wait for one another at grid barriers;
 * every such wait gives up after a bounded number of spins, and the call
 * that launched it returns HC_ERR_TIMEOUT with the context still usable (hc_run
 * then redoes the recomputation first thing in its next call).  spins > 0
 * sets that bound (0 restores the built-in ones) and makes each barrier
 * expect extra_arrivals more blocks than were launched, so that every wait
 * runs out: the way the tests check this path without a fault. */
hc_status hc_test_bounded_waits(hc_ctx* ctx, int32_t spins, int32_t extra_arrivals);

/* Launch-shape autotuner (no counterpart in the reference).  hc_run times
 * k_flow_route's launch shapes (register budget, grid, and the face-compacted
 * variant of the kernel) on the live state
 * the first time a context reaches a shape class (erosion terms, Manning's n
 * field, wet-list length to a power of two; below 65,536 wet cells the
 * default shape is kept) and caches the fastest per class for the process.
 * The timing launches leave the model state as it was.  force != 0 times
 * them now; *shape (optional) receives the shape in use, ms (optional, n
 * doubles) the last timings per shape in ms per launch. */
hc_status hc_autotune(hc_ctx* ctx, int32_t force, int32_t* shape, double* ms, int32_t n);
/* Fixes k_flow_route's launch shape (0 .. 17; every shape computes the same
 * results), or -1: back to the autotuner. */
hc_status hc_set_launch_shape(hc_ctx* ctx, int32_t shape);

/* Stream the context issues its work on (a cudaStream_t). */
void* hc_stream(hc_ctx* ctx);

/* Measurement hook (no counterpart in the reference): launches one kernel of
 * the path `reps` times on the current state between two CUDA events on the
 * context's stream and returns the mean time per launch in ms.  `kernel` is
 * "flow_route", "depth_update", "scan_area" or "entrain".  The launches
 * change the state like real calls would.  *wet receives the number of cells
 * in the wet mask. */
hc_status hc_bench_kernel(hc_ctx* ctx, const char* kernel, int32_t reps, double* avg_ms,
                          int64_t* wet);

/* Measurement hook (no counterpart in the reference): kernels this context
 * has launched (graph kernel nodes included) and bytes it has copied
 * host->device and device->host, since hc_create. */
hc_status hc_get_counters(hc_ctx* ctx, int64_t* launches, int64_t* h2d_bytes,
                          int64_t* d2h_bytes);

/* Measurement hook (no counterpart in the reference): runs one iteration of
 * hc_run's sequence phase by phase, without the graph, timing each phase with
 * CUDA events: ms[0..8] = control+inputs, flow_route, depth_update,
 * scan_area, entrainment passes, apply and lateral passes with the edge
 * output, lateral3, water_flux_out, slide_3 (device time; the host's reads
 * of the control block between passes are in no phase). */
hc_status hc_profile_iteration(hc_ctx* ctx, int32_t flags, double* ms);

#ifdef __cplusplus
}
#endif
#endif
