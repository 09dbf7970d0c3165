// Hydraulic part of one iteration: the driver's scalar logic (timestep,
// counters, water inputs, TOPMODEL), flow_route, depth_update, scan_area and
// water_flux_out.
//
// Reference: src/catchmentmodel/LSDCatchmentModel.cpp (line numbers below)
// and src/main.cpp:139-204.  Every expression that produces model state keeps
// the reference's operand order and roundings (the library is compiled with
// --fmad=false, so nothing is contracted into an FMA unless written so): the
// hydraulic state is bit-identical to the reference's serial build.

#include "hc_internal.cuh"

#include <math.h>
#include <algorithm>

namespace {

constexpr double kG = 9.81;  // gravity, LSDCatchmentModel.hpp:438

__device__ __forceinline__ double cfl_dt(const hc_params& p, double maxdepth) {
  // courant_friedrichs_lewy_condition :1884-1887
  return p.courant_number * (p.DX / sqrt(kG * (maxdepth)));
}

__device__ __forceinline__ double flow_dt_of(const hc_params& p, const hc_scalars& s) {
  // get_flow_timestep :1913-1923
  double f = s.time_step;
  double c = cfl_dt(p, s.maxdepth);
  if (f > c) f = c;
  return f;
}

// ---------------------------------------------------------------------------
// control: set_loop_cycle .. catchment_waterinputs (main.cpp:142-158), one
// thread.  Also decides which members run in this iteration.
// ---------------------------------------------------------------------------
__device__ void topmodel_step(hc_dev* d, const hc_params& p, const double* topm, int rows) {
  // topmodel_runoff(time_1) :3649-3715: the recurrence depends only on the
  // rain table, so the host evaluates it once (host_topmodel_table) and the
  // device steps through the rows.
  int t = (int)d->s.time_1;
  const int rf = p.rfnum;
  if (t < 0 || t >= rows) {
    d->err_code = 101;
    d->pause |= HC_PAUSE_ERROR;
    return;
  }
  const double* row = topm + (size_t)t * 2 * (rf + 1);
  for (int n = p.spatially_complex_rainfall ? 0 : 1; n <= rf; n++) {
    d->s.old_j_mean[n] = row[n];
    d->s.new_j_mean[n] = row[(rf + 1) + n];
  }
}

__global__ void k_control(const hc_view c, hc_dev* d, hc_iter_handles hh) {
  const hc_params& p = c.p;
  hc_scalars& s = d->s;
  if (d->pause || d->budget <= 0) {
    // skipped iteration: every gated kernel of it returns at once; the
    // switches of the iteration that paused stay as they are, for the host
    // to finish that iteration
    if (d->budget <= 0) d->pause |= HC_PAUSE_BUDGET;
    d->it_active = 0;
    return;
  }
  d->do_scan = d->do_erode = d->do_slide = d->do_lateral = 0;
  d->erode_retry = 0;
  d->erode_passes = 0;
  d->budget--;
  d->it_active = 1;
  d->rest_active = 1;

  s.previous = s.cycle;                                   // set_loop_cycle :1873
  s.input_output_difference = fabs(s.waterinput - s.waterOut);  // :1879
  if (s.maxdepth <= 0.1) s.maxdepth = 0.1;                // set_maximum_timestep :1890
  if (s.time_step < cfl_dt(p, s.maxdepth)) s.time_step = cfl_dt(p, s.maxdepth);
  if (s.input_output_difference > p.in_out_difference_allowed &&
      s.time_step > (cfl_dt(p, s.maxdepth)))
    s.time_step = cfl_dt(p, s.maxdepth);
  // adjoint runs record the time steps, or impose recorded ones
  const bool adj = c.adj_dt && d->adj_mode && d->adj_i < d->adj_n;
  double* arec = adj ? c.adj_dt + (size_t)d->adj_i * HC_ADJ_REC : nullptr;
  if (adj) {
    if (d->adj_mode == 2) s.time_step = arec[0];
    else arec[0] = s.time_step;
  }
  s.counter += 1;                                         // increment_counters :1925
  s.cycle += s.time_step / 60;

  const double DX = p.DX;
  // reach_water_and_sediment_input :3301-3452
  if (p.reach_mode) {
    const double fdt = flow_dt_of(p, s);
    const int rdt = p.reach_input_data_timestep;
    const int div = p.div_inputs;
    const int row = (int)(s.cycle / rdt);
    if (!p.hydro_only) {
      for (int n = 0; n <= p.number_of_points - 1; n++) {
        const int x = p.inpoints[n][0], y = p.inpoints[n][1];
        const size_t cell = (size_t)x * c.W + y;
        double adding_factor = 1, added_tot = 0;
        if (c.h[cell] > p.water_depth_erosion_threshold) {
          const float* r = c.reach[n] + (size_t)row * c.reach_cols[n];
          for (int tn = 5; tn <= HC_G + 3; tn++) {
            float q = fabsf(r[tn]) / div;  // float / int in the reference
            added_tot += q / (DX * DX) / (rdt * 60) * s.time_step;
          }
          if (added_tot / p.number_of_points > p.ERODEFACTOR * 0.75)
            adding_factor = (p.ERODEFACTOR * 0.75) / (added_tot / p.number_of_points);
          if (c.index[cell] == -9999) {  // addGS :3949, serial position: now
            d->grain_tot++;
            c.index[cell] = d->grain_tot;
            grain_record_init(c, cell, c.elev[cell], c.bed[cell]);
          }
          for (int tn = 5; tn <= HC_G + 3; tn++) {
            double amt = adding_factor * (double)fabsf(r[tn]) / div / (DX * DX) / (rdt * 60) *
                         s.time_step;
            if (p.isSuspended[tn - 4]) {
              c.vs[cell] += amt;
            } else {
              grain_at(c, cell, tn - 4) += amt;
              c.elev[cell] += amt;
            }
          }
        }
      }
    }
    for (int n = 0; n <= p.number_of_points - 1; n++) {
      const int x = p.inpoints[n][0], y = p.inpoints[n][1];
      const size_t cell = (size_t)x * c.W + y;
      if (row + 1 >= c.reach_rows[n]) {
        d->err_code = 102;
        d->pause |= HC_PAUSE_ERROR;
        continue;
      }
      double i1 = c.reach[n][(size_t)row * c.reach_cols[n] + 1];
      double i2 = c.reach[n][(size_t)(row + 1) * c.reach_cols[n] + 1];
      double prop = (((row + 1) * rdt) - s.cycle) / rdt;
      double input = i1 + ((i2 - i1) * (1 - prop));
      s.waterinput += (input / div);
      const double add = (input / div) / (DX * DX) * fdt;
      c.h[cell] += add;
      if (x >= 1 && x <= c.imax && y >= 1 && y <= c.jmax) d->vin_step += add;
    }
  }

  // catchment_waterinputs :2027 -> catchment_water_input_and_hydrology :3455
  s.waterinput = 0;
  double fdt2 = flow_dt_of(p, s);
  if (adj) {
    if (d->adj_mode == 2) fdt2 = arec[1];
    else arec[1] = fdt2;
  }
  if (p.spatially_complex_rainfall) {
    // catchment_water_input_and_hydrology(flow_timestep, runoff) :3544-3607.
    // A cell's runoff recurrence (runoffGrid::calculate_runoff) depends only
    // on its rain, i.e. on its rain state: the zone (zones 1 .. rfnum-1, or
    // column 0 for all cells when rfnum is 1) or none (state 0: zone rfnum
    // and others get no rain, rainGrid::create, LSDRainfallRunoff.cpp:33-66),
    // so every cell of a state holds the
    // same values; the host tabulates them per state with glibc.
    const int rf = p.rfnum;
    for (int z = 0; z <= rf; z++) {
      double amt = s.j_mean[z] * fdt2;
      if (amt > p.ERODEFACTOR) amt = p.ERODEFACTOR;
      d->input_amt[z] = amt;
      d->j_mean_in[z] = s.j_mean[z];
    }
    // the two sums over the cells (:3547-3571), formed state by state
    for (int z = 0; z <= rf; z++) s.waterinput += c.runoff_count[z] * (s.j_mean[z] * DX * DX);
    for (int z = 0; z <= rf; z++)
      s.waterinput += c.runoff_count[z] * ((d->input_amt[z] / fdt2) * DX * DX);
    // ledger: k_runoff_inputs adds input_amt[z] to each computed cell of state z
    for (int z = 0; z <= rf; z++)
      if (c.runoff_count[z] > 0) d->vin_step += c.runoff_count[z] * d->input_amt[z];
    d->input_dt = fdt2;
    // new_jmeanmax (:3575-3586), over the states that hold a computed cell
    double jmm = 0;
    for (int z = 0; z <= rf; z++)
      if (((c.runoff_present >> z) & 1u) && s.new_j_mean[z] > jmm) jmm = s.new_j_mean[z];
    if (s.cycle >= s.time_1) {
      do {
        s.time_1++;
        topmodel_step(d, p, c.topm, c.topm_rows);
        if (s.time_step > p.max_time_step &&
            jmm > (0.2 / ((unsigned)p.jmax * (unsigned)p.imax * DX * DX))) {
          s.cycle = s.time_1 + (p.max_time_step / 60);
          s.time_step = p.max_time_step;
        }
      } while (s.time_1 < s.cycle && !(d->pause & HC_PAUSE_ERROR));
    }
    for (int z = 0; z <= rf; z++)  // calchydrograph(time, runoff) :3728-3740
      s.j_mean[z] = s.old_j_mean[z] + (((s.new_j_mean[z] - s.old_j_mean[z]) / 2) *
                                       (2 - (s.time_1 - s.cycle)));
    d->do_drain = 0;  // no drainage area or input points in this mode
  } else {
    for (int i = 1; i <= p.rfnum; i++) s.waterinput += s.j_mean[i] * s.nActualGridCells[i] * DX * DX;
    for (int i = 0; i <= p.rfnum; i++) d->j_mean_in[i] = s.j_mean[i];
    if (arec)
      for (int i = 0; i <= HC_MAX_RF; i++) arec[3 + i] = (i <= p.rfnum) ? s.j_mean[i] : 0.0;
    d->input_dt = fdt2;
    // what each input point of a zone receives (:3463-3477), the same for all
    // points of the zone
    for (int z = 0; z <= p.rfnum && z <= HC_MAX_RF; z++) {
      double amt = (d->j_mean_in[z] * s.nActualGridCells[z]) / (s.catchment_input_counter[z]) * fdt2;
      if (amt > p.ERODEFACTOR) amt = p.ERODEFACTOR;
      d->input_amt[z] = amt;
    }
    if (s.cycle >= s.time_1) {
      do {
        s.time_1++;
        topmodel_step(d, p, c.topm, c.topm_rows);
        if (s.time_step > p.max_time_step) {
          double jmm = 0;
          for (int n = 1; n <= p.rfnum; n++)
            if (s.new_j_mean[n] > jmm) jmm = s.new_j_mean[n];
          if (jmm > (0.2 / ((unsigned)p.imax * (unsigned)p.jmax * DX * DX))) {
            s.cycle = s.time_1 + (p.max_time_step / 60);
            s.time_step = p.max_time_step;
          }
        }
      } while (s.time_1 < s.cycle && !(d->pause & HC_PAUSE_ERROR));
    }
    for (int n = 1; n <= p.rfnum; n++)  // calchydrograph :3718
      s.j_mean[n] = s.old_j_mean[n] + (((s.new_j_mean[n] - s.old_j_mean[n]) / 2) * (2 - (s.time_1 - s.cycle)));
    if (arec) {
      arec[HC_ADJ_T1] = s.time_1;
      arec[HC_ADJ_T1 + 1] = s.cycle;
    }
    double jmeanmax = 0;
    for (int n = 1; n <= p.rfnum; n++)
      if (s.j_mean[n] > jmeanmax) jmeanmax = s.j_mean[n];
    bool recalc = false;
    if (jmeanmax >= s.baseflow) {
      s.baseflow = s.baseflow * 3;
      recalc = true;
    }
    if (s.baseflow > (jmeanmax * 3) && s.baseflow > 0.000001) {
      s.baseflow = jmeanmax * 1.25;
      recalc = true;
    }
    // The drainage area and the input-point list are recomputed before the
    // next iteration (the host sorts the elevations, hc_drain.cu does the
    // rest), from the elevations as they are now (k_depth_update copies
    // them before the iteration's erosion); the
    // reference, too, applies the new list from the next iteration on.
    d->do_drain = recalc;
    if (recalc) d->pause |= HC_PAUSE_DRAINAGE;
  }

  s.flow_timestep = flow_dt_of(p, s);
  if (adj) {
    if (d->adj_mode == 2) s.flow_timestep = arec[2];
    else arec[2] = s.flow_timestep;
    d->adj_i++;
  }
  d->do_scan = ((long long)s.counter % p.scan_area_interval_iter) == 0;
  d->do_erode = !p.hydro_only && s.counter >= s.erode_call;
  d->erode_retry = d->do_erode;
  if (d->do_erode) {
    // erode()'s start (:4219; k_erode_begin for a direct call): the
    // kernels between here and the erosion block read flow_timestep, set
    // above, not time_step
    s.time_step = s.time_step * 1.5;
    d->mult = s.erode_mult;
    d->tempbmax_bits = 0;
  }
  d->do_slide = !p.hydro_only && ((long long)s.counter % p.in_channel_landslide_iter_interval) == 0;
  if (hh.has) {
    // kernels inside the bodies enabled here: scan 3, erosion 5 + 7, slide_3 4
    d->body_kernels += (d->do_scan ? 3 : 0) + (d->do_erode && !p.hydro_only ? 12 : 0) +
                       (d->do_slide ? 4 : 0);
    cudaGraphSetConditional(hh.scan, d->do_scan ? 1u : 0u);
    if (!p.hydro_only) {
      cudaGraphSetConditional(hh.erode, d->do_erode ? 1u : 0u);
      cudaGraphSetConditional(hh.erode_fin, d->do_erode ? 1u : 0u);
      cudaGraphSetConditional(hh.slide, d->do_slide ? 1u : 0u);
    }
  }
}

// catchment input points (:3463-3477): one thread per point
// The ledger counts what lands on the grid (rows 1..imax, columns 1..jmax):
// with no point found the reference still visits one (totalinputpoints
// forced to 1, :3765), whose coordinates may be stale or the padding corner.
__global__ void k_inputs(const hc_view c, hc_dev* d) {
  if (!d->it_active) return;
  const hc_scalars& s = d->s;
  const int total = (int)s.totalinputpoints;
  double added = 0;
  for (int z = 1 + blockIdx.x * blockDim.x + threadIdx.x; z <= total;
       z += gridDim.x * blockDim.x) {
    const int i = c.cin_x[z], j = c.cin_y[z];
    const size_t cell = (size_t)i * c.W + j;
    const double a = d->input_amt[c.rfarea[cell]];
    c.h[cell] += a;
    if (i >= 1 && i <= c.imax && j >= 1 && j <= c.jmax) added += a;
  }
  double tot;
  if (grid_sum(added, c.vpart, &d->sum_done, &tot)) d->vin_step += tot;
}

// Distributed runoff (:3560-3573): every computed cell (rows 1 .. imax-1,
// columns 1 .. jmax-1, elevation above no-data) takes its state's amount.
__global__ void k_runoff_inputs(const hc_view c, hc_dev* d) {
  if (!d->it_active) return;
  const int j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int i = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= c.imax || j >= c.jmax) return;
  const size_t cell = (size_t)i * c.W + j;
  if (!(dkey(c.elev[cell]) > kNoDataKey)) return;  // j_mean stays 0 there
  const int rf = c.p.rfnum, r = c.rfarea[cell];
  const int z = (rf == 1) ? 1 : ((r >= 1 && r <= rf - 1) ? r : 0);
  c.h[cell] += d->input_amt[z];
}

__global__ void k_flow_dt(const hc_view c, hc_dev* d) {
  d->s.flow_timestep = flow_dt_of(c.p, d->s);
  d->it_active = 1;
  d->rest_active = 1;
}

// ---------------------------------------------------------------------------
// flow_route :3063-3247.  One thread per cell; cells outside the wet mask keep
// their discharges (the reference does not visit them).
// ---------------------------------------------------------------------------
struct FaceOut {
  double q, qs, vel;
  int dir;  // 1: positive, -1: negative, 0: none
};

// The limiters' FP64 tests, for the faces whose float estimates cannot
// decide them: out of line, so that their FP64 instructions (a hardware
// division among them) issue only where they run.
static __device__ __noinline__ bool depth_exceeds(double qn, double dt, double DX, double h) {
  return (qn * dt / DX) > (h / 4);  // :3138, :3218
}
static __device__ __noinline__ bool depth_exceeds_neg(double qn, double dt, double DX, double h) {
  return fabs(qn * dt / DX) > (h / 4);  // :3144, :3219
}
static __device__ __noinline__ bool sed_exceeds(double qs, double dt, double v, double DX) {
  return qs * dt > (v * DX) / 4;  // :3163
}
static __device__ __noinline__ bool sed_exceeds_neg(double qs, double dt, double v, double DX) {
  return fabs(qs * dt) > (v * DX) / 4;  // :3169
}

// The limiters' replacement values and the Froude test's exact form, out of
// line as well: they run for few faces, and inlined, their integer-pipe
// divisions and square roots would double the kernel's code, whose
// instruction fetches stall the warps more than anything else.
// (x * DX / 5) / dt, the depth and sediment limits' value (:3140, :3165)
static __device__ __noinline__ double limit_value(double x, double DX, double dt) {
  return ddiv_rn(ddiv_rn(x * DX, 5.0), dt);
}
// |q/hflow| / sqrt(g hflow) > froude_limit, exactly (:3124)
static __device__ __noinline__ bool froude_exceeds(double qoh, double hflow, double fl) {
  return dgt(ddiv_rn(fabs(qoh), isqrt_rn(kG * hflow)), fl);
}
// hflow * (sqrt(g hflow) * froude_limit), the Froude limit's value (:3127)
static __device__ __noinline__ double froude_value(double hflow, double fl) {
  return hflow * (isqrt_rn(kG * hflow) * fl);
}

// Three-way test of A > B from float estimates a, b, each within a relative
// 2^-18 of A, B (or flushed to 0 below 2^-126, inf above the float range):
// +1 surely greater, -1 surely not, 0 too close to call (the caller then
// evaluates the reference's FP64 expression).  Tiny pairs, where a flushed
// estimate carries no relative bound, are never decided here.
__device__ __forceinline__ int decide_gt(float a, float b) {
  const float m = 1e-4f * (fabsf(a) + fabsf(b));
  if (!(m >= 1e-34f) || !(m < 1e30f)) return 0;
  const float dd = a - b;
  if (dd > m) return 1;
  if (dd < -m) return -1;
  return 0;
}

// One face of the inertial scheme (:3096-3191 / :3193-3242).  e0,h0: this
// cell; e1,h1: the upstream neighbour (x-1 for qx, y-1 for qy); a0, a1 the
// water surfaces e+h.  `edge_slope` is 0 for interior faces, +1 / -1 where
// the reference replaces the slope by +/-edgeslope.
//
// The FP64 pipe (1.2 TFLOP/s on GB300) bounds this kernel, and compares
// occupy it as much as arithmetic does.  So every test runs on the integer
// pipe (dgt0, dlt, ...: IEEE results for non-NaN operands), and the limiter
// tests, which only pick a branch, are first decided on float estimates; the
// reference's FP64 expression is evaluated only when the estimate is within
// 1e-4 of the threshold.  The branch taken - and so the result - is always
// the reference's.
// The face past the hflow gate: hflow (> hflow_threshold) and dA = a1 - a0
// (the surface difference) as the gate formed them.
// The face update's divisions: inline, or (kCall) through one out-of-line
// copy, which keeps the kernel's code small (its instruction fetches stall
// the warps) at the cost of a call per division; a launch-shape choice of
// the face-compacted kernel.
static __device__ __noinline__ double ddiv_rn_call(double a, double b) { return ddiv_rn(a, b); }
template <bool kCall>
__device__ __forceinline__ double fdiv(double a, double b) {
  if (kCall) return ddiv_rn_call(a, b);
  return ddiv_rn(a, b);
}

template <bool kSusp, bool kVel, bool kCall = false>
__device__ __forceinline__ void inertial_face_core(double& q, double& qs, double& vel_out,
                                                   int& vdir, double hflow, double dA, double h0,
                                                   double h1, double v0, double v1, double c0,
                                                   double nn, double dt, int edge_slope,
                                                   const hc_view& c) {
  const hc_params& p = c.p;
  const double DX = p.DX;
  vdir = 0;
  double slope = ddiv_by(dA, c.dxd);
  if (edge_slope == 1) slope = p.edgeslope;
  if (edge_slope == -1) slope = zero_minus(p.edgeslope);
  const double ghd = kG * hflow * dt;
  // the numerator once for both branches (a branch apiece would issue its
  // FP64 instructions twice in a warp that holds both)
  double qn = q - (ghd * slope);
  // q = 0: (0 - ghd*slope) / (1 + (ghd*nn*0)/h^3) = (0 - ghd*slope) / 1
  if (!deq0(q)) {
    const double aq = __longlong_as_double(dbits(q) & 0x7fffffffffffffffLL);  // fabs
    qn = fdiv<kCall>(qn, 1 + fdiv<kCall>(ghd * nn * aq, icube_rn(hflow)));
  }
  const float hf = approx_abs_f(hflow);
  const float dtf = approx_abs_f(dt);
  // q/hflow: exact when the face velocity is kept (erosion runs), where it
  // also serves the Froude test
  double qoh = 0;
  bool qoh_valid = false;
  // Froude limit: |q/hflow| / sqrt(g*hflow) > froude_limit
  if (!deq0(qn)) {
    float fr;
    if (kVel) {
      qoh = fdiv<kCall>(qn, hflow);
      qoh_valid = true;
      fr = approx_abs_f(qoh) / sqrtf(9.81f * hf);
    } else {
      fr = approx_abs_f(qn) / (hf * sqrtf(9.81f * hf));
    }
    int t = decide_gt(fr, c.flf);
    if (t == 0) {
      if (!qoh_valid) qoh = fdiv<kCall>(qn, hflow);
      t = froude_exceeds(qoh, hflow, p.froude_limit) ? 1 : -1;
    }
    if (t > 0) {
      const double lim = froude_value(hflow, p.froude_limit);
      qn = dgt0(qn) ? lim : zero_minus(lim);
      qoh_valid = false;
    }
  }
  // depth limit: |q*dt/DX| > (depth of the giving cell)/4; the two tests
  // run one after the other, as in the reference
  if (dgt0(qn)) {
    int t = decide_gt(approx_abs_f(qn) * dtf / c.DXf, approx_f(h0) * 0.25f);
    if (t == 0) t = depth_exceeds(qn, dt, DX, h0) ? 1 : -1;
    if (t > 0) {
      qn = limit_value(h0, DX, dt);
      qoh_valid = false;
    }
  }
  if (dlt0(qn)) {
    int t = decide_gt(approx_abs_f(qn) * dtf / c.DXf, approx_f(h1) * 0.25f);
    if (t == 0) t = depth_exceeds_neg(qn, dt, DX, h1) ? 1 : -1;
    if (t > 0) {
      qn = zero_minus(limit_value(h1, DX, dt));
      qoh_valid = false;
    }
  }
  const bool qpos = dgt0(qn), qneg = dlt0(qn);
  if (kSusp) {
    // qs = q * (V/h) of the giving cell; V = 0 gives 0 * q (a signed zero)
    // (one product for both signs: h1 > 0 here, as h0 above)
    if (qpos || qneg) qs = qn * (qpos ? c0 : (deq0(v1) ? v1 : fdiv<kCall>(v1, h1)));
    // qs*dt > V*DX/4 (giving cell) caps the sediment flux
    if (dgt0(qs)) {
      int t = decide_gt(approx_abs_f(qs) * dtf, approx_f(v0) * c.DXf * 0.25f);
      if (t == 0) t = sed_exceeds(qs, dt, v0, DX) ? 1 : -1;
      if (t > 0) qs = limit_value(v0, DX, dt);
    }
    if (dlt0(qs)) {
      int t = decide_gt(approx_abs_f(qs) * dtf, approx_f(v1) * c.DXf * 0.25f);
      if (t == 0) t = sed_exceeds_neg(qs, dt, v1, DX) ? 1 : -1;
      if (t > 0) qs = zero_minus(limit_value(v1, DX, dt));
    }
  }
  if (kVel) {
    // (0 - q)/hflow = -(q/hflow) exactly: division rounds symmetrically
    if ((qpos || qneg) && !qoh_valid) qoh = fdiv<kCall>(qn, hflow);
    if (qpos) {
      vel_out = qoh;
      vdir = 1;
    }
    if (qneg) {
      vel_out = zero_minus(qoh);
      vdir = -1;
    }
  }
  q = qn;
}

template <bool kSusp, bool kVel>
__device__ __forceinline__ void inertial_face(double& q, double& qs, double& vel_out, int& vdir,
                                              double e0, double h0, double a0, double e1,
                                              double h1, double a1, double v0, double v1,
                                              double c0, double nn, double dt, int edge_slope,
                                              const hc_view& c) {
  vdir = 0;
  double hflow = imax_d(a0, a1) - imax_d(e1, e0);
  if (!(dkey(hflow) > c.thr_key)) {  // hflow > hflow_threshold
    q = 0;
    qs = 0;
    return;
  }
  inertial_face_core<kSusp, kVel>(q, qs, vel_out, vdir, hflow, a1 - a0, h0, h1, v0, v1, c0, nn,
                                  dt, edge_slope, c);
}

template <bool kSed>
__device__ __forceinline__ void flow_cell(const hc_view& c, const hc_dev* __restrict__ d,
                                          size_t cell) {
  const size_t W = c.W, N2 = c.N2;
  const int i = (int)(cell / W), j = (int)(cell % W);
  const double e0 = c.elev[cell];
  // e > -9999 (no-data and below are skipped)
  auto above_nodata = [](double e) { return dkey(e) > kNoDataKey; };
  if (!above_nodata(e0)) return;
  const hc_params& p = c.p;
  const double dt = d->s.flow_timestep;
  const double n = p.spatially_var_mannings ? c.man[cell] : p.mannings;
  const double nn = n * n;
  const bool susp = kSed && p.isSuspended[1] != 0;
  const double h0 = c.h[cell];
  const double a0 = e0 + h0;
  const double v0 = susp ? c.vs[cell] : 0.0;
  // V/h of this cell, shared by both faces.  Only used where q > 0 after
  // the depth limit, which implies h > 0, so a zero V gives V itself (with
  // its sign) without the division.
  const double c0 = (susp && !deq0(v0)) ? ddiv_rn(v0, h0) : v0;
  const bool wet0 = dgt0(h0);
  // x face (rows i-1, i)
  {
    const size_t up = cell - W;
    const double h1 = c.h[up], e1 = c.elev[up];
    if ((wet0 || dgt0(h1)) && above_nodata(e1)) {
      double q = c.qx[cell], qs = kSed ? c.qxs[cell] : 0.0, vel = 0;
      int vdir;
      const int es = (i == c.imax) ? 1 : ((i <= 2) ? -1 : 0);
      if (susp)
        inertial_face<true, kSed>(q, qs, vel, vdir, e0, h0, a0, e1, h1, e1 + h1, v0, c.vs[up],
                                  c0, nn, dt, es, c);
      else
        inertial_face<false, kSed>(q, qs, vel, vdir, e0, h0, a0, e1, h1, e1 + h1, v0, 0.0, c0,
                                   nn, dt, es, c);
      c.qx[cell] = q;
      if (kSed) {
        c.qxs[cell] = qs;
        if (vdir == 1) c.vd[3 * N2 + cell] = vel;  // vel_dir[x][y][7]
        if (vdir == -1) c.vd[1 * N2 + up] = vel;   // vel_dir[x-1][y][3]
      }
    }
  }
  // y face (columns j-1, j).  The reference takes max(e0, e1) with the
  // operands the other way round (:3197-3198); for ordered values max is
  // symmetric, so one face routine serves both.
  {
    const size_t lf = cell - 1;
    const double h1 = c.h[lf], e1 = c.elev[lf];
    if ((wet0 || dgt0(h1)) && above_nodata(e1)) {
      double q = c.qy[cell], qs = kSed ? c.qys[cell] : 0.0, vel = 0;
      int vdir;
      const int es = (j == c.jmax) ? 1 : ((j <= 2) ? -1 : 0);
      if (susp)
        inertial_face<true, kSed>(q, qs, vel, vdir, e0, h0, a0, e1, h1, e1 + h1, v0, c.vs[lf],
                                  c0, nn, dt, es, c);
      else
        inertial_face<false, kSed>(q, qs, vel, vdir, e0, h0, a0, e1, h1, e1 + h1, v0, 0.0, c0,
                                   nn, dt, es, c);
      c.qy[cell] = q;
      if (kSed) {
        c.qys[cell] = qs;
        if (vdir == 1) c.vd[0 * N2 + cell] = vel;  // vel_dir[x][y][1]
        if (vdir == -1) c.vd[2 * N2 + lf] = vel;   // vel_dir[x][y-1][5]
      }
    }
  }
}

// One thread per wet cell, grid-stride over the wet list: cells outside the
// mask are never touched, as in the reference's down_scan loops.  MINB,
// the blocks of 256 a multiprocessor must hold, sets the register budget
// (3: 80 registers, 4: 64, 5: 48, 6: 40; the autotuner picks one).
template <bool kSed, int MINB>
__global__ void __launch_bounds__(256, MINB) k_flow_route(const hc_view c,
                                                          const hc_dev* __restrict__ d, int gated) {
  if (gated && !d->it_active) return;
  const int n = d->wet_count;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    flow_cell<kSed>(c, d, (size_t)c.wet[k]);
}

// Face-compacted flow_route.  In a storm about half the listed cells are dry
// and two faces in three fail the gate (both cells dry) or the hflow
// threshold, so a warp evaluating its 32 cells' faces in turn issues the
// FP64 instructions of a face with a third of its lanes.  Here each lane
// first classifies its cell's two faces (the gate and hflow: two additions
// and compares) and writes q = qs = 0 for gated faces below the threshold;
// the faces that go on are queued in the warp's shared-memory queue (cell,
// face, hflow, a1 - a0), and whenever 32 are queued the warp evaluates them
// together, one per lane, the rest carried over to the next cells.  Every
// face is evaluated from the same inputs by the same expressions as in
// k_flow_route, so the results are the same bit for bit.
constexpr int kFaceQ = 96;  // queue entries per warp: < 32 carried + 64 new

template <bool kSed, bool kCall>
__device__ __forceinline__ void face_work(const hc_view& c, const hc_dev* __restrict__ d,
                                          uint32_t f, double hflow, double dA, double dt) {
  const size_t W = c.W, N2 = c.N2;
  const size_t cell = f >> 1;
  const bool yface = f & 1u;
  const size_t nb = yface ? cell - 1 : cell - W;
  const int i = (int)(cell / W), j = (int)(cell - (size_t)i * W);
  const hc_params& p = c.p;
  const double n = p.spatially_var_mannings ? c.man[cell] : p.mannings;
  const double nn = n * n;
  const bool susp = kSed && p.isSuspended[1] != 0;
  const double h0 = c.h[cell], h1 = c.h[nb];
  const double v0 = susp ? c.vs[cell] : 0.0;
  const double c0 = (susp && !deq0(v0)) ? fdiv<kCall>(v0, h0) : v0;
  double* qa = yface ? c.qy : c.qx;
  double* qsa = yface ? c.qys : c.qxs;
  double q = qa[cell], qs = kSed ? qsa[cell] : 0.0, vel = 0;
  int vdir;
  const int es = yface ? ((j == c.jmax) ? 1 : ((j <= 2) ? -1 : 0))
                       : ((i == c.imax) ? 1 : ((i <= 2) ? -1 : 0));
  if (susp)
    inertial_face_core<true, kSed, kCall>(q, qs, vel, vdir, hflow, dA, h0, h1, v0, c.vs[nb], c0, nn,
                                   dt, es, c);
  else
    inertial_face_core<false, kSed, kCall>(q, qs, vel, vdir, hflow, dA, h0, h1, v0, 0.0, c0, nn, dt,
                                    es, c);
  qa[cell] = q;
  if (kSed) {
    qsa[cell] = qs;
    // x face: vel_dir[x][y][7] / vel_dir[x-1][y][3]; y face: [x][y][1] / [x][y-1][5]
    if (vdir == 1) c.vd[(yface ? 0 : 3) * N2 + cell] = vel;
    if (vdir == -1) c.vd[(yface ? 2 : 1) * N2 + nb] = vel;
  }
}

template <bool kSed, int MINB, bool kCall = false>
__global__ void __launch_bounds__(256, MINB) k_flow_route_q(const hc_view c,
                                                            const hc_dev* __restrict__ d,
                                                            int gated) {
  __shared__ uint32_t qf[8][kFaceQ];
  __shared__ double qh[8][kFaceQ], qa[8][kFaceQ];
  if (gated && !d->it_active) return;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* Q = qf[warp];
  double* HF = qh[warp];
  double* DA = qa[warp];
  const int n = d->wet_count;
  const double dt = d->s.flow_timestep;
  const size_t W = c.W;
  const int warps = gridDim.x * (blockDim.x >> 5);
  int qn = 0;  // the same on every lane
  // the list entry of the warp's next turn is fetched a turn ahead (its
  // cell's loads then need not wait for it)
  int base = (blockIdx.x * (blockDim.x >> 5) + warp) * 32;
  uint32_t next = (base + lane < n) ? (uint32_t)c.wet[base + lane] : 0u;
  for (; base < n; base += warps * 32) {
    const int k = base + lane;
    bool fx = false, fy = false;
    double hx = 0, hy = 0, ax = 0, ay = 0;
    uint32_t cell = 0;
    const uint32_t mine = next;
    if (k + warps * 32 < n) next = (uint32_t)c.wet[k + warps * 32];
    if (k < n) {
      cell = mine;
      const double e0 = c.elev[cell];
      if (dkey(e0) > kNoDataKey) {  // e > -9999
        const double h0 = c.h[cell];
        const double a0 = e0 + h0;
        const bool wet0 = dgt0(h0);
        {
          const size_t up = cell - W;
          const double h1 = c.h[up], e1 = c.elev[up];
          if ((wet0 || dgt0(h1)) && dkey(e1) > kNoDataKey) {
            const double a1 = e1 + h1;
            hx = imax_d(a0, a1) - imax_d(e1, e0);
            ax = a1 - a0;
            fx = dkey(hx) > c.thr_key;
            if (!fx) {
              c.qx[cell] = 0;
              if (kSed) c.qxs[cell] = 0;
            }
          }
        }
        {
          const size_t lf = cell - 1;
          const double h1 = c.h[lf], e1 = c.elev[lf];
          if ((wet0 || dgt0(h1)) && dkey(e1) > kNoDataKey) {
            const double a1 = e1 + h1;
            hy = imax_d(a0, a1) - imax_d(e1, e0);
            ay = a1 - a0;
            fy = dkey(hy) > c.thr_key;
            if (!fy) {
              c.qy[cell] = 0;
              if (kSed) c.qys[cell] = 0;
            }
          }
        }
      }
    }
    const unsigned bx = __ballot_sync(FULL, fx), by = __ballot_sync(FULL, fy);
    const unsigned below = (1u << lane) - 1u;
    const int nx = __popc(bx);
    if (fx) {
      const int s = qn + __popc(bx & below);
      Q[s] = cell << 1;
      HF[s] = hx;
      DA[s] = ax;
    }
    if (fy) {
      const int s = qn + nx + __popc(by & below);
      Q[s] = (cell << 1) | 1u;
      HF[s] = hy;
      DA[s] = ay;
    }
    qn += nx + __popc(by);
    __syncwarp();
    while (qn >= 32) {
      qn -= 32;
      const uint32_t f = Q[qn + lane];
      const double hf = HF[qn + lane], da = DA[qn + lane];
      __syncwarp();  // the entries are read before the next cells' are written
      face_work<kSed, kCall>(c, d, f, hf, da, dt);
    }
  }
  if (lane < qn) face_work<kSed, kCall>(c, d, Q[lane], HF[lane], DA[lane], dt);
}

// ---------------------------------------------------------------------------
// depth_update :3259-3299 with the maxdepth reduction (warp shuffle, block,
// then the last block publishes the grid result).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 6) k_depth_update(const hc_view c, hc_dev* d, int gated) {
  __shared__ long long warp_max[8];
  __shared__ bool last;
  if (gated && !d->it_active) return;
  const size_t W = c.W;
  const double dt = d->s.flow_timestep;
  const bool susp = c.p.isSuspended[1] && !c.p.hydro_only;
  const int nw = d->wet_count;
  // the running maximum is kept as the bits of a non-negative double, which
  // order like the values; tests run on the integer pipe (dgt0 etc.)
  long long m = 0;
  bool nonfinite = false;
  double lost = 0;  // water zeroed at no-data cells (the ledger's `lost`)
  // The ledger's mask-edge term: a face between a listed cell and one
  // outside the wet list changes only the listed cell's depth (the other is
  // not updated), so the water crossing it appears or vanishes.  The same
  // expression as the update, over those faces only.
  double edge = 0;
  // The discharges, fluxes, mask, border and elevations are not written by
  // this kernel: they are read through the read-only path (__ldg).  The next
  // list entry is fetched a turn ahead, so that its cell's loads do not wait
  // for the index behind them.
  const int stride = gridDim.x * blockDim.x;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  int next = (k < nw) ? __ldg(c.wet + k) : 0;
  for (; k < nw; k += stride) {
    const size_t cell = (size_t)next;
    if (k + stride < nw) next = __ldg(c.wet + k + stride);
    if (__ldg(c.border + cell)) {  // k_wet_write marks the listed cells on the border
      const uint8_t mu = __ldg(c.mask + cell - W), md = __ldg(c.mask + cell + W),
                    ml = __ldg(c.mask + cell - 1), mr = __ldg(c.mask + cell + 1);
      const double ux1 = md ? 0.0 : __ldg(c.qx + cell + W), ux0 = mu ? 0.0 : __ldg(c.qx + cell);
      const double uy1 = mr ? 0.0 : __ldg(c.qy + cell + 1), uy0 = ml ? 0.0 : __ldg(c.qy + cell);
      edge += ddiv_by(dt * (ux1 - ux0 + uy1 - uy0), c.dxd);
    }
    // Where the four fluxes are zero (either sign) the update adds a signed
    // zero, which leaves any value but -0 as it is: the FP64 work is skipped
    // then (dry pockets of the list; cells without suspended load).
    constexpr long long kNegZero = (long long)0x8000000000000000ULL;
    double h = c.h[cell];
    {
      const double a = __ldg(c.qx + cell + W), b = __ldg(c.qx + cell),
                   e = __ldg(c.qy + cell + 1), f = __ldg(c.qy + cell);
      if (((dbits(a) | dbits(b) | dbits(e) | dbits(f)) << 1) != 0 || dbits(h) == kNegZero)
        h += ddiv_by(dt * (a - b + e - f), c.dxd);
    }
    // hydro-only runs keep Vsusptot at zero (no sediment source exists)
    if (susp) {
      const double a = __ldg(c.qxs + cell + W), b = __ldg(c.qxs + cell),
                   e = __ldg(c.qys + cell + 1), f = __ldg(c.qys + cell);
      const double v = c.vs[cell];
      if (((dbits(a) | dbits(b) | dbits(e) | dbits(f)) << 1) != 0 || dbits(v) == kNegZero)
        c.vs[cell] = v + ddiv_by(dt * (a - b + e - f), c.dxd);
    }
    nonfinite |= disnan(h);
    if (dgt0(h)) {
      if (dbits(__ldg(c.elev + cell)) == kNoDataBits) {
        lost += h;
        h = 0;
      } else {
        m = max(m, dbits(h));
      }
    }
    c.h[cell] = h;
  }
  // no flux enters a no-data cell, so this is empty in practice (its order
  // of addition is not fixed)
  // the elevations the drainage recomputation after this iteration starts
  // from (flow and depth_update leave them unchanged; erosion comes later);
  // only erosion runs keep the copy (hydro-only elevations never change)
  if (gated && d->do_drain && c.drain_snap)
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < c.N2;
         k += (size_t)gridDim.x * blockDim.x)
      c.drain_snap[k] = c.elev[k];
  if (!deq0(lost)) atomicAdd(&d->vlost_step, lost);
  if (nonfinite) {
    d->err_code = 301;  // a NaN water depth: the run cannot continue
    atomicOr((unsigned int*)&d->pause, HC_PAUSE_ERROR);
  }
  const double esum = block_sum(edge);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  const int t = threadIdx.x;
  if ((t & 31) == 0) warp_max[t >> 5] = m;
  __syncthreads();
  if (t == 0) {
    long long b = 0;
    for (int w = 0; w < (int)blockDim.x / 32; w++) b = max(b, warp_max[w]);
    if (b > 0) atomicMax(&d->maxdepth_bits, (unsigned long long)b);
    c.vpart[blockIdx.x] = esum;
    __threadfence();
    last = (atomicAdd(&d->depth_done, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    // the blocks' mask-edge sums, added in block order
    double a = 0;
    for (int k = t; k < (int)gridDim.x; k += blockDim.x) a += ((volatile double*)c.vpart)[k];
    const double etot = block_sum(a);
    if (t == 0) {
      unsigned long long bits = atomicExch(&d->maxdepth_bits, 0ull);
      d->s.maxdepth = __longlong_as_double((long long)bits);
      d->maxdepth_step = d->s.maxdepth;
      d->vmask_step += etot;
      d->depth_done = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// scan_area :3821-3849 (every scan_area_interval_iter iterations)
// ---------------------------------------------------------------------------
// Also the ledger's volume: the depth sum of its block (rows 1..imax,
// columns 1..jmax) into vpart, added up in order by k_wet_count's last block.
__global__ void __launch_bounds__(256) k_scan_area(const hc_view c, const hc_dev* __restrict__ d,
                                                    int gated) {
  if (gated && !(d->it_active && d->do_scan)) return;
  const int j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int i = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  double v = 0;
  if (i <= c.imax && j <= c.jmax) {
    const size_t W = c.W;
    const size_t cell = (size_t)i * W + j;
    const double* h = c.h;
    v = h[cell];
    bool wet = v > 0 || h[cell - 1] > 0 || h[cell + 1] > 0 || h[cell - W] > 0 ||
               h[cell - W - 1] > 0 || h[cell - W + 1] > 0 || h[cell + W - 1] > 0 ||
               h[cell + W + 1] > 0 || h[cell + W] > 0;
    c.mask[cell] = wet ? 1 : 0;
  }
  const double bsum = block_sum(v);
  if (threadIdx.x == 0 && threadIdx.y == 0) c.vpart[blockIdx.x + blockIdx.y * gridDim.x] = bsum;
}

// The wet list: mask bytes counted per block of 1024 cells, the counts
// scanned, the cell numbers written in ascending order.
// The block counts, then, in the block that finishes last, their exclusive
// scan (the wet list's offsets per block) and the list's length.  nvol:
// blocks of the k_scan_area launch before it, whose volume partials the same
// block adds up (0: none, the list is rebuilt from a mask kept as it was).
__global__ void __launch_bounds__(1024) k_wet_count(const hc_view c, hc_dev* d, int gated,
                                                    int nvol) {
  __shared__ int ws[32];
  if (gated && !(d->it_active && d->do_scan)) return;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int v = (i < c.N2) ? c.mask[i] : 0;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < 32; k++) s += ws[k];
    c.wet_sums[blockIdx.x] = s;
  }
  if (!last_to_arrive(&d->wet_arrive)) return;
  if (nvol > 0) {
    double a = 0;
    for (int k = threadIdx.x; k < nvol; k += blockDim.x) a += c.vpart[k];
    const double tot = block_sum(a);
    if (threadIdx.x == 0) {
      d->vol_scan = tot;
      d->vol_scan_counter = d->s.counter;
    }
  }
  const int total = scan_block_counts(c.wet_sums, (int)gridDim.x);
  if (threadIdx.x == 0) d->wet_count = total;
}

__global__ void __launch_bounds__(1024) k_wet_write(const hc_view c, const hc_dev* d, int gated) {
  __shared__ int ws[32], wb[32];
  if (gated && !(d->it_active && d->do_scan)) return;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int v = (i < c.N2) ? c.mask[i] : 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < 32; k++) {
      wb[k] = s;
      s += ws[k];
    }
  }
  __syncthreads();
  if (v) c.wet[c.wet_sums[blockIdx.x] + wb[warp] + incl - 1] = (int32_t)i;
  // the wet list's border (listed cells are in rows 1..imax, columns
  // 1..jmax, so their four neighbours lie inside the padded grid)
  if (i < c.N2)
    c.border[i] = v && !(c.mask[i - 1] && c.mask[i + 1] && c.mask[i - c.W] && c.mask[i + c.W]);
}

// ---------------------------------------------------------------------------
// water_flux_out :3005-3047, one block.  Each edge cell is clamped at its
// first visit in the reference's loop order; the outflow sum is a fixed-order
// tree (deterministic, equal to the serial sum up to rounding).
// Also writes the iteration record and the end-of-loop test of main.cpp:204.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_flux_out(const hc_view c, hc_dev* d, int gated, int record,
                                                    hc_step_record* rec, int64_t rec_cap) {
  __shared__ double part[1024];
  __shared__ double vpart[1024];
  if (gated && !(d->it_active && d->rest_active)) return;
  const hc_params& p = c.p;
  const int imax = c.imax, jmax = c.jmax;
  const double thr = p.water_depth_erosion_threshold, DX = p.DX;
  const double fdt = d->s.time_step;
  const int n1 = 2 * imax, n2 = n1 + 2 * jmax;
  double acc = 0, vacc = 0;  // the outflow rate, and the depth taken off
  for (int k = threadIdx.x; k < n2; k += blockDim.x) {
    int i, j;
    if (k < n1) {
      i = 1 + k / 2;
      if ((k & 1) == 0) {
        j = jmax;
      } else {
        j = 1;
        if (jmax == 1) continue;  // same cell as the right-hand edge
      }
    } else {
      const int kk = k - n1;
      j = 1 + kk / 2;
      if (j == 1 || j == jmax) continue;  // already visited by the row loop
      if ((kk & 1) == 0) {
        i = 1;
      } else {
        i = imax;
        if (imax == 1) continue;
      }
    }
    double& h = c.h[(size_t)i * c.W + j];
    if (h > thr) {
      acc += (h - thr) * DX * DX / fdt;
      vacc += h - thr;
      h = thr;
    }
  }
  part[threadIdx.x] = acc;
  vpart[threadIdx.x] = vacc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      part[threadIdx.x] += part[threadIdx.x + w];
      vpart[threadIdx.x] += vpart[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    hc_scalars& s = d->s;
    s.temptot = part[0];
    s.waterOut = s.temptot;
    if (record && rec && d->rec_index < rec_cap) {
      hc_step_record& r = rec[d->rec_index];
      r.counter = s.counter;
      r.cycle = s.cycle;
      r.time_step = s.time_step;
      r.maxdepth = d->maxdepth_step;
      r.waterOut = s.waterOut;
      r.waterinput = s.waterinput;
      r.erode_mult = s.erode_mult;
      r.sediQ = s.sediQ;
      r.globalsediq = s.globalsediq;
      r.baseflow = s.baseflow;
      const double a2 = DX * DX;
      r.vol_in = d->vin_step * a2;
      r.vol_out = (vpart[0] + d->vlost_step) * a2;
      r.vol_mask = d->vmask_step * a2;
      r.volume = (d->vol_scan_counter == s.counter) ? d->vol_scan * a2 : __longlong_as_double(0x7ff8000000000000LL);
    }
    if (record) d->rec_index++;
    if (gated) d->wet_steps += (unsigned long long)d->wet_count;
    // the ledger: this iteration's terms join the totals
    d->vin_tot += d->vin_step;
    d->vout_tot += vpart[0];
    d->vlost_tot += d->vlost_step;
    d->vmask_tot += d->vmask_step;
    d->vin_step = 0;
    d->vlost_step = 0;
    d->vmask_step = 0;
    if (gated) {
      if (!p.hydro_only && !(d->flags & HC_RUN_NOHILL) &&
          (s.cycle > s.creep_time || s.cycle > s.creep_time2))
        d->pause |= HC_PAUSE_HOSTSTEP;
      if (!(s.cycle / 60 < p.maxcycle)) d->pause |= HC_PAUSE_FINISHED;
    }
  }
}

// The depth sum of the grid (rows 1..imax, columns 1..jmax) now, in a fixed
// order (hc_mass_balance; the ledger's start).
__global__ void __launch_bounds__(256) k_volume(const hc_view c, hc_dev* d) {
  const size_t n = (size_t)c.imax * c.jmax;
  double a = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t i = 1 + k / c.jmax, j = 1 + k % c.jmax;
    a += c.h[i * c.W + j];
  }
  double tot;
  if (grid_sum(a, c.vpart, &d->sum_done, &tot)) d->vol_now = tot;
}

__global__ void k_mass_reset(hc_dev* d) {
  d->vol0 = d->vol_now;
  d->vin_tot = d->vout_tot = d->vlost_tot = d->vmask_tot = 0;
  d->vin_step = d->vlost_step = d->vmask_step = 0;
}

}  // namespace

// ------------------------------------------------------------------ launches
static dim3 grid2d(const hc_ctx* c, dim3 b) {
  return dim3((c->v.jmax + b.x - 1) / b.x, (c->v.imax + b.y - 1) / b.y);
}

void launch_control(hc_ctx* c) {
  k_control<<<1, 1, 0, c->cs>>>(c->v, c->dev, c->hcur);
  count_launch(c, 1);
}

void launch_inputs(hc_ctx* c) {
  if (c->v.p.spatially_complex_rainfall) {
    dim3 b(32, 8), g((c->v.jmax + 31) / 32, (c->v.imax + 7) / 8);
    k_runoff_inputs<<<g, b, 0, c->cs>>>(c->v, c->dev);
    count_launch(c, 1);
    return;
  }
  // grid-stride over the current list (its length lives on the device):
  // four blocks per SM on large grids, fewer on small ones, whose lists are
  // short (ensembles run many small members' launches side by side)
  int n = c->v.cin_cap;
  const int cap = std::min(c->sms * 4, std::max(c->sms, (int)(c->v.N2 / 4096)));
  int blocks = std::min((n + 255) / 256, std::min(cap, c->v.vpart_cap));
  if (blocks < 1) blocks = 1;
  k_inputs<<<blocks, 256, 0, c->cs>>>(c->v, c->dev);
  count_launch(c, 1);
}

void launch_flow_dt(hc_ctx* c) {
  k_flow_dt<<<1, 1, 0, c->cs>>>(c->v, c->dev);
  count_launch(c, 1);
}

// grid-stride kernels over the wet list: enough blocks to fill the GPU, no
// more (the list length lives on the device)
static int list_blocks(const hc_ctx* c) {
  const size_t need = (c->v.N2 + 255) / 256;
  return (int)std::min<size_t>(need, 152 * 8);
}

// The launch shapes of k_flow_route the autotuner chooses from: blocks per
// multiprocessor (the register budget) and waves of the grid (grid = SMs x
// blocks per SM x waves; one wave: every block resident at once).
const FlowShape kFlowShapes[kFlowShapeCount] = {
    {4, 0, 0}, {3, 1, 0}, {4, 1, 0}, {5, 1, 0}, {6, 1, 0}, {3, 4, 0}, {4, 4, 0}, {5, 4, 0},
    {6, 4, 0}, {3, 1, 1}, {4, 1, 1}, {5, 1, 1}, {3, 4, 1}, {4, 4, 1}, {5, 4, 1},
    {3, 1, 2}, {4, 1, 2}, {5, 1, 2}};

template <bool kSed>
static void flow_launch(hc_ctx* c, int gated, int shape) {
  const FlowShape f = kFlowShapes[shape];
  int blocks = f.waves ? c->sms * f.minb * f.waves : list_blocks(c);
  blocks = std::max(1, std::min(blocks, (int)((c->v.N2 + 255) / 256)));
  if (f.compact == 2) {  // divisions through one out-of-line copy
    switch (f.minb) {
      case 3: k_flow_route_q<kSed, 3, true><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
      case 5: k_flow_route_q<kSed, 5, true><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
      default: k_flow_route_q<kSed, 4, true><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
    }
    return;
  }
  if (f.compact) {
    switch (f.minb) {
      case 3: k_flow_route_q<kSed, 3><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
      case 5: k_flow_route_q<kSed, 5><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
      default: k_flow_route_q<kSed, 4><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
    }
    return;
  }
  switch (f.minb) {
    case 3: k_flow_route<kSed, 3><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
    case 5: k_flow_route<kSed, 5><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
    case 6: k_flow_route<kSed, 6><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
    default: k_flow_route<kSed, 4><<<blocks, 256, 0, c->cs>>>(c->v, c->dev, gated); break;
  }
}

void launch_flow_route_shape(hc_ctx* c, int gated, int shape) {
  if (shape < 0 || shape >= kFlowShapeCount) shape = 0;
  if (c->v.p.hydro_only) flow_launch<false>(c, gated, shape);
  else flow_launch<true>(c, gated, shape);
  count_launch(c, 1);
}

void launch_flow_route(hc_ctx* c, int gated) { launch_flow_route_shape(c, gated, c->flow_shape); }

void launch_depth_update(hc_ctx* c, int gated) {
  k_depth_update<<<list_blocks(c), 256, 0, c->cs>>>(c->v, c->dev, gated);
  count_launch(c, 1);
}

static void wet_list(hc_ctx* c, int gated, int nvol);

void launch_scan_area(hc_ctx* c, int gated) {
  dim3 b(32, 8);
  const dim3 g = grid2d(c, b);
  k_scan_area<<<g, b, 0, c->cs>>>(c->v, c->dev, gated);
  count_launch(c, 1);
  wet_list(c, gated, (int)(g.x * g.y));
}

void launch_wet_list(hc_ctx* c, int gated) { wet_list(c, gated, 0); }

static void wet_list(hc_ctx* c, int gated, int nvol) {
  const int nb = (int)((c->v.N2 + 1023) / 1024);
  k_wet_count<<<nb, 1024, 0, c->cs>>>(c->v, c->dev, gated, nvol);
  k_wet_write<<<nb, 1024, 0, c->cs>>>(c->v, c->dev, gated);
  count_launch(c, 2);
}

void launch_flux_out(hc_ctx* c, int gated, int record) {
  k_flux_out<<<1, 1024, 0, c->cs>>>(c->v, c->dev, gated, record, c->v.rec, c->v.rec_cap);
  count_launch(c, 1);
}

// grid of the grid_sum kernels: at most the SMs x 4 blocks of 256 (the
// partials array holds vpart_cap entries)
static int sum_blocks(const hc_ctx* c, size_t n) {
  const size_t need = (n + 255) / 256;
  return (int)std::max<size_t>(1, std::min<size_t>(need, (size_t)std::min(152 * 4, c->v.vpart_cap)));
}

void launch_volume(hc_ctx* c) {
  k_volume<<<sum_blocks(c, (size_t)c->v.imax * c->v.jmax), 256, 0, c->cs>>>(c->v, c->dev);
  count_launch(c, 1);
}

void launch_mass_reset(hc_ctx* c) {
  launch_volume(c);
  k_mass_reset<<<1, 1, 0, c->cs>>>(c->dev);
  count_launch(c, 1);
}
