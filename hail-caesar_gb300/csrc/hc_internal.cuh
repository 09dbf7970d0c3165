// Internal definitions of libhc_gpu (not part of the C ABI).
//
// Device layout of the model state (all in HBM, resident for the whole run):
//   padded 2-D fields: (imax+2) x (jmax+2) doubles, row pitch W = jmax+2,
//                      the reference's TNT layout, so whole-field transfers
//                      are single copies;
//   vel_dir:           4 planes (directions 1,3,5,7 of the reference's
//                      9-entry cell record; the other 5 are never used);
//   sr/sl/su/sd:       4 x 10 planes, plane (dir, fraction);
//   grain, strata:     one record slot per cell (SoA planes, 11 and 10x9),
//                      instead of the reference's lazily numbered rows; the
//                      reference's row numbers (index[][]) are still kept,
//                      allocated in the reference's serial order, and
//                      hc_download(HC_F_GRAIN/STRATA) writes rows by them;
//   mask:              one byte per cell, 1 where the cell is in down_scan.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include <utility>

#include "../../include/hc_gpu.h"

#define HC_G 10               // G_MAX
#define HC_NFRAC 9            // fractions 1..9
#define HC_ST_N 9             // strata fractions used (0..G_MAX-2)

// pause reasons (hc_dev::pause)
#define HC_PAUSE_NONE 0
#define HC_PAUSE_DRAINAGE 1   // baseflow changed: host recomputes input points
#define HC_PAUSE_ERODE 2      // erosion retry loop exceeded the in-graph passes
#define HC_PAUSE_FINISHED 4   // cycle/60 >= maxcycle
#define HC_PAUSE_BUDGET 8     // iteration budget of the current hc_run reached
#define HC_PAUSE_ERROR 16     // device-side error (see err_code)
#define HC_PAUSE_HOSTSTEP 32  // host-side step due (creep / global landsliding)
#define HC_PAUSE_LATERAL 64   // lateral3 due (runs before water_flux_out)

#define HC_ERODE_PASSES 4     // entrainment passes captured per iteration

// per-iteration record of an adjoint run: [0] time_step after
// set_maximum_timestep, [1] the input points' dt, [2] the flow dt,
// [3 .. 3+HC_MAX_RF] j_mean as the input points used it, then time_1 and
// cycle as calchydrograph used them
#define HC_ADJ_REC (3 + HC_MAX_RF + 1 + 2)
#define HC_ADJ_T1 (3 + HC_MAX_RF + 1)
static_assert(HC_ADJ_REC == HC_ADJ_RECORD, "record size of the C ABI");

// Device-side control block.  One per context, in device memory; the single
// thread control kernel owns the scalar logic of the reference's driver.
struct hc_dev {
  hc_scalars s;           // scalar model state (mirrors LSDCatchmentModel)
  // per-iteration switches written by the control kernel
  int it_active;          // this iteration runs
  int do_scan;            // scan_area this iteration
  int do_erode;           // erosion this iteration
  int erode_retry;        // another entrainment pass is needed
  int erode_passes;       // passes done in this erosion call
  int rest_active;        // kernels after the entrainment passes run
  int do_slide;           // in_channel_landsliding this iteration
  int do_lateral;         // lateral3 this iteration
  int pause;              // HC_PAUSE_* bits; set -> following iterations skip
  int err_code;
  int64_t budget;         // iterations left in the current hc_run
  int64_t rec_index;      // next record slot
  double maxdepth_step;   // maxdepth right after depth_update (for records)
  double reach_dt;        // flow dt used by the water inputs this iteration
  double j_mean_in[HC_MAX_RF + 1];  // j_mean used by the input points
  double input_dt;        // flow dt used by the catchment input points
  double input_amt[HC_MAX_RF + 1];  // water each input point of a zone receives
  double mult;            // mult_factor of the current erode() call
  unsigned long long maxdepth_bits;  // atomic max of h (positive doubles)
  unsigned long long tempbmax_bits;  // atomic max of temptot1
  int grain_tot;          // grain_array_tot as an int
  int alloc_count;        // allocations pending in the current pass
  int flags;              // HC_RUN_* of the current run
  unsigned int depth_done;   // blocks finished in depth_update (last-block reduction)
  unsigned int pass_done;    // blocks finished in an entrainment pass
  unsigned int misc_done;
  // arrival counters of the launches whose last block finishes the step
  // (last_to_arrive): the wet list's count, the grain records' count and
  // assignment, slide_3's flag count; each is zero between launches
  unsigned int wet_arrive, alloc_arrive, assign_arrive, flag_arrive;
  unsigned long long body_kernels;  // kernels run inside conditional graph nodes
  int wet_count;          // length of hc_view::wet
  int do_drain;           // this iteration moved the baseflow threshold
  unsigned int drain_front, drain_done, drain_points, drain_levels;
  unsigned int drain_rf[HC_MAX_RF + 1];
  int adj_mode;           // 0 off, 1 record the time steps, 2 impose them
  int64_t adj_i, adj_n;   // next iteration, capacity of hc_view::adj_dt
  int64_t adj_slot_t0, adj_slot_n;  // iterations whose state k_adj_save keeps
  double *adj_slot_h, *adj_slot_qx, *adj_slot_qy;  // ... and where (slot k at k * N2)
  uint8_t *adj_slot_mask;
  unsigned int xchains;   // chain starts of the +/-x apply pass (hc_view::chains)
  unsigned int ychains;   // chain starts of the +/-y apply pass
  unsigned int xresume, yresume;  // long chains handed from the thread to the warp walkers
  unsigned int xtake, ytake;      // chains taken so far by the thread walkers
  unsigned int ent_n;     // cells listed for the transport of an entrainment pass
  // water ledger, as sums of water depth (m; times DX^2 gives m^3)
  double vin_step;        // added by the inputs since the last water_flux_out
  double vlost_step;      // zeroed by depth_update at no-data cells, likewise
  double vmask_step;      // crossed faces between a listed and an unlisted cell, likewise
  double vin_tot, vout_tot, vlost_tot, vmask_tot;  // since the ledger started
  double vol0;            // depth sum of the grid when the ledger started
  double vol_scan;        // depth sum of the grid at the last scan_area
  double vol_scan_counter;  // the iteration (counter) of that scan_area
  double vol_now;         // depth sum of the grid, written by k_volume
  unsigned int sum_done;  // blocks finished in a grid_sum (left at zero)
  unsigned long long wet_steps;  // wet-list length summed over the iterations run
};

// Working state of a drainage recomputation (hc_drain.cu): the radix
// selection of the sweep's last reached position and the checks that decide
// whether the sort's tie order can matter.
struct hc_drain_aux {
  unsigned long long prefix, mask, k, gt, real_eq;  // selection of the P-th largest
  unsigned long long min_u;                         // smallest elevation key
  unsigned int min_count, min_matters, contrib_tie, pad;
  unsigned int hist[256];
};

// A divisor prepared for ddiv_by (below): its significand, exponent and a
// 64-bit reciprocal of the significand.
struct hc_divisor {
  unsigned long long mb, V;  // significand of b, ~2^116/mb (unused when mb == 2^52)
  double b;
  int eb;                    // biased exponent of b
  int ok;                    // b normal and finite
};

// Everything a kernel needs, passed by value (device pointers + parameters).
struct hc_view {
  hc_params p;
  double rDX;             // RN(1/DX) (the adjoint's slope derivatives)
  hc_divisor dxd;         // DX as a divisor (ddiv_by)
  float DXf, flf;         // DX and froude_limit as floats (estimates only)
  float act_hi, act_lo;   // (float)(active*1.5), (float)(active/4): sort_active's estimates
  long long thr_key;      // dkey(hflow_threshold)
  int imax, jmax;
  size_t W, N2, E2;       // pitch, padded cells, edge-array cells

  // fields
  double *elev, *h, *qx, *qy, *qxs, *qys, *vs, *vel, *tau, *bed, *man, *area, *ss;
  double *vd;        // 4 * N2
  double *sflux;     // 4 dirs * 10 fractions * N2 ; dir order su, sr, sd, sl
  uint8_t *sdirty;   // N2: 1 where the cell's sflux entries may be nonzero
  double *grain;     // 12 * N2: a cell's fractions side by side (grain_at)
  double *strata;    // 90 * N2: a cell's 10 layers x 9 fractions side by side (strata_at)
  int32_t *index;
  uint8_t *mask;
  uint8_t *border;   // N2: 1 where a listed cell has an unlisted 4-neighbour (wet-list border)
  int32_t *rfarea;
  double *edge, *edge2, *veg;  // E2, E2, 4*E2 (reference layout)
  int32_t *cin_x, *cin_y;      // catchment input points (1-based lists)
  int32_t *wet;                // cells of the wet mask, ascending (the down_scan
                               // lists as one array); length in hc_dev::wet_count
  int32_t *wet_sums;           // per-block counts for building it
  uint32_t *ent_list;          // cells with flow in an entrainment pass (N2)
  double *ent_qs;              // their qtot and slope sum (2 per entry)
  int cin_cap;

  // time series
  float *rain; int rain_rows, rain_cols;
  float *reach[HC_MAX_POINTS]; int reach_rows[HC_MAX_POINTS], reach_cols[HC_MAX_POINTS];
  double *topm; int topm_rows;   // precomputed TOPMODEL recurrence
  double dlog[HC_G];             // log(d1..d9) for d50
  // Einstein per-fraction constants, evaluated on the host with the
  // reference's expressions (:4393-4394): (2650-1000)*Di, the square root
  // sqrt(1000/((2250-1000)*g*Di^3)) and its reciprocal
  double runoff_count[HC_MAX_RF + 1];  // distributed runoff: computed cells per rain state
  unsigned runoff_present;             // bit z: rain state z holds a computed cell
  double einA[HC_G], einS[HC_G];
  hc_divisor einSd[HC_G];  // the einS as divisors

  // scratch
  double *erodetot, *erodetot3;  // N2 each
  double *pre;                   // 12 * N2: per-cell apply-pass terms, side by side (PRE)
  uint32_t *chains;              // 4 * N2: apply-pass chain starts (x pass, y pass), then
                                 // the resume points of long chains (x, y)
  // drainage area (hc_drain.cu): sweep position, sum of drops, higher
  // neighbours pending, two frontiers, and the elevation snapshot
  uint32_t *drain_pos, *drain_f0, *drain_f1;
  int32_t *drain_pend;
  double *drain_dt, *drain_snap;
  double *drain_frac;     // 9*N2: share of neighbour k's area pushed here (plane k)
  uint16_t *drain_multi;  // N2: neighbours (bit k) that push here in more than one direction
  struct hc_drain_aux *drain_aux;
  // adjoint runs (hc_adjoint.cu): per-iteration time steps, recorded or
  // imposed (HC_ADJ_REC stride per iteration; see hc_dev::adj_mode)
  double *adj_dt;
  // adjoint replay: set while the graphs carry k_adj_save, which keeps each
  // iteration's state before it in the slot set that hc_dev::adj_slot_*
  // names (slot = iteration - hc_dev::adj_slot_t0)
  double *adj_sh, *adj_sqx, *adj_sqy;
  uint8_t *adj_smask;
  unsigned long long *alloc_key; // N2: serial-order key of the first grain-record request
  int32_t *alloc_list;           // N2: cells allocated, in order
  int32_t *slide_list; int slide_cap;
  uint8_t *touched;              // N2 bytes
  double *red;                   // reduction scratch
  int32_t *scan_tmp;             // scan scratch
  double *vpart; int vpart_cap;  // per-block partial sums (grid_sum, scan_area's volume)
  hc_step_record *rec; int64_t rec_cap;
  // test hook of the bounded device waits (hc_test_bounded_waits): when
  // wait_spins > 0 the drainage sweep's waits give up after that many spins,
  // and its grid barrier expects barrier_extra arrivals more than there are
  // blocks (with no single-block frontiers), so that every wait runs out
  int wait_spins, barrier_extra;
};

// Conditional-node handles of one captured iteration (CUDA graph IF nodes):
// the control kernel and the entrainment passes set them, so steps that are
// not due this iteration are not launched at all.
struct hc_iter_handles {
  cudaGraphConditionalHandle scan, erode, retry2, retry3, retry4, erode_fin, slide;
  int has;  // 0 outside graph capture: nothing to set
};

constexpr int kMaxFlowShapes = 24;  // launch shapes of k_flow_route the tuner can time

struct hc_ctx {
  hc_view v;
  cudaStream_t s;         // the context's stream
  cudaStream_t cs;        // stream launches go to (a side stream while a
                          // conditional node's body is captured)
  cudaStream_t s2;
  cudaStream_t s3;         // snapshots to host memory (hc_snapshot_begin)
  hc_iter_handles hcur;   // handles of the iteration being captured
  int device;
  char err[512];
  size_t bytes, max_bytes;
  hc_dev *dev;       // device control block
  hc_dev *hdev;      // pinned host mirror
  double *h_elev;    // pinned host buffer (drainage area)
  bool prepared;
  // host copy of the catchment input list (kept between recomputations, as
  // the reference keeps its vector)
  int32_t *h_cin_x, *h_cin_y;
  void* drainage_cache;    // sweep order of the drainage area, reused while elev is unchanged
  struct hc_sort_work* sort_work;  // device sort of the elevations (hc_sort.cu)
  bool area_valid;         // device area matches the cached sweep order
  bool drain_retry;        // a drainage recomputation gave up: redo it first
  int sms;                 // multiprocessors of the device
  int flow_shape;          // launch shape of k_flow_route (kFlowShapes), autotuned
  bool flow_pinned;        // the caller fixed flow_shape (hc_set_launch_shape)
  int64_t tuned_key;       // the shape class flow_shape was chosen for (-1: none)
  double tune_ms[kMaxFlowShapes];  // the autotuner's times per shape (ms per launch)
  // called after every recomputation of the input points (adjoint replays)
  void (*points_hook)(hc_ctx*, void*);
  void* points_hook_arg;
  // CUDA graph of K iterations
  cudaGraphExec_t graph; int graph_iters; int graph_flags;
  int64_t graph_kernels;   // kernel nodes in the graph
  // graphs of 2^k iterations (k < 12) for runs shorter than a chunk, made
  // when first needed: a short run takes the fewest launches (20 = 16 + 4)
  cudaGraphExec_t tail[12];
  int64_t tail_kernels[12];
  int chunk_pref;          // iterations per chunk graph asked for (0: the default)
  int chunk_iters;         // iterations in the chunk last launched
  cudaEvent_t chunk_done;  // a launched chunk and its control-block copy are done
  int64_t run_n;           // iterations asked of the current run
  unsigned long long body_k0;
  int64_t budget0;         // budget when the current chunk was launched
  bool capturing;
  // counters for measurement: kernels launched, bytes moved host<->device
  int64_t launches, h2d_bytes, d2h_bytes;
  // hc_run statistics (HC_STAT_*): how often each kind of host work ran and
  // the host wall time it took
  int64_t stat_n[HC_STAT_COUNT];
  double stat_ms[HC_STAT_COUNT];
};

inline void count_launch(hc_ctx* c, int n) {
  if (!c->capturing) c->launches += n;
}

// ---------------------------------------------------------------- helpers
#define HC_DEV __device__ __forceinline__

// Sum of one double per thread over the block, in a fixed order (warp
// shuffles, then the warps in order); the result is valid in thread 0.
// Every thread of the block calls it; blockDim a multiple of 32, <= 1024.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[32];
  // a warp whose values are all +0 sums to +0: no FP64 adds (sums of
  // sparse terms, like the ledger's border fluxes, are mostly such warps)
  if (__ballot_sync(0xffffffffu, __double_as_longlong(v) != 0))
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int t = threadIdx.x + threadIdx.y * blockDim.x;
  const int nw = (blockDim.x * blockDim.y) >> 5;
  __syncthreads();  // ws may still be read by a previous call
  if ((t & 31) == 0) ws[t >> 5] = v;
  __syncthreads();
  double s = 0;
  if (t == 0)
    for (int w = 0; w < nw; w++) s += ws[w];
  return s;
}

// Called once by every block of a launch (all its threads), after the
// block's own writes: true in every thread of the block that arrives last,
// which then sees every block's writes (read them through volatile or
// __ldcg: L1 is not coherent); the counter is back at zero afterwards.
__device__ __forceinline__ bool last_to_arrive(unsigned int* counter) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x * gridDim.y - 1;
    if (last) *counter = 0;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// Exclusive prefix sums, in place, of the per-block counts sums[0..n)
// written by the blocks of the same launch, by one block of 1024 threads;
// returns the total (in every thread).
__device__ __forceinline__ int scan_block_counts(int32_t* sums, int n) {
  __shared__ int buf[1024];
  __shared__ int carry;
  volatile int32_t* vs = sums;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int k = base + threadIdx.x;
    const int v = (k < n) ? vs[k] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const int t = (threadIdx.x >= (unsigned)off) ? buf[threadIdx.x - off] : 0;
      __syncthreads();
      buf[threadIdx.x] += t;
      __syncthreads();
    }
    if (k < n) vs[k] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
  return carry;
}

// Deterministic grid-wide sum: each block stores its block_sum in part[b];
// the last block to finish adds part[0..blocks) in a fixed order (thread t
// takes t, t+bs, ...; then block_sum) and returns true in its thread 0 with
// the total in *out.  *done is left at zero.  Every thread of every block
// calls it.
__device__ __forceinline__ bool grid_sum(double v, double* part, unsigned int* done,
                                         double* out) {
  __shared__ bool last;
  const int t = threadIdx.x + threadIdx.y * blockDim.x;
  const int bs = blockDim.x * blockDim.y;
  const unsigned nb = gridDim.x * gridDim.y;
  const unsigned b = blockIdx.x + blockIdx.y * gridDim.x;
  const double s = block_sum(v);
  if (t == 0) {
    part[b] = s;
    __threadfence();
    last = (atomicAdd(done, 1u) == nb - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double a = 0;
  for (unsigned k = t; k < nb; k += bs) a += ((volatile double*)part)[k];
  const double tot = block_sum(a);
  if (t == 0) {
    *out = tot;
    *done = 0;
  }
  return t == 0;
}

// std::max(a, b) as libstdc++ defines it: (a < b) ? b : a
HC_DEV double smax(double a, double b) { return (a < b) ? b : a; }

// Comparisons of doubles on the integer pipe.  On this GPU a compare,
// like any FP64-pipe instruction, costs the issue slots of dozens of
// integer instructions, and the stencils are FP64-pipe bound.  Results are
// the IEEE ones for every operand that is not a NaN, with +0 == -0.
HC_DEV long long dbits(double x) { return __double_as_longlong(x); }
// monotone key: x < y  <=>  dkey(x) < dkey(y); dkey(+0) == dkey(-0) == 0
HC_DEV long long dkey(double x) {
  const long long b = dbits(x);
  const long long s = b >> 63;
  return ((b & 0x7fffffffffffffffLL) ^ s) - s;
}
HC_DEV bool dgt0(double x) { return dbits(x) > 0; }                     // x > 0
HC_DEV bool dlt0(double x) { return dbits(x) < 0 && (dbits(x) << 1) != 0; }  // x < 0
HC_DEV bool deq0(double x) { return (dbits(x) << 1) == 0; }             // x == 0
HC_DEV bool dlt(double a, double b) { return dkey(a) < dkey(b); }       // a < b
HC_DEV bool dgt(double a, double b) { return dkey(a) > dkey(b); }       // a > b
constexpr long long kNoDataKey = -0x40C3878000000000LL;  // dkey(-9999.0)
constexpr long long kNoDataBits = (long long)0xC0C3878000000000ULL;  // dbits(-9999.0)
// smax on the integer pipe
HC_DEV double imax_d(double a, double b) { return dlt(a, b) ? b : a; }
// 0 - x (the reference's spelling of a negation: +0 for x = +0)
HC_DEV double zero_minus(double x) {
  return deq0(x) ? 0.0 : __longlong_as_double(dbits(x) ^ (long long)0x8000000000000000ULL);
}
// x is a NaN
HC_DEV bool disnan(double x) {
  return (dbits(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}

// h^3 rounded to nearest.  The reference evaluates std::pow(hflow, 10/3),
// i.e. pow(hflow, 3.0) in C++11, which glibc returns correctly rounded in
// all but vanishingly rare cases.  Here: exact h^2 = p + e (two-product),
// h^3 = p*h + e*h with p*h split exactly again, summed once.
HC_DEV double cube_rn(double h) {
  double p = __dmul_rn(h, h);
  double e = fma(h, h, -p);
  double q = __dmul_rn(p, h);
  double f = fma(p, h, -q);
  double c = fma(e, h, f);
  return __dadd_rn(q, c);
}

// h^3 rounded to nearest-even, computed exactly on the integer pipe: the
// cube of the 53-bit significand m (159 bits, from two 64x64 products) is
// rounded at its 53rd bit with the round bit and a sticky bit, the exponent
// is 3E plus the normalisation shift.  Five FP64 instructions (cube_rn)
// occupy this GPU's FP64 pipe for as long as about 150 integer ones; this
// takes about 45.  Zero, subnormal, infinite or NaN h, and cubes outside
// the normal range, take cube_rn.
// (a call, so that the compiler does not if-convert it: predicated-off FP64
// instructions still take their issue slots on the FP64 pipe)
static __device__ __noinline__ double cube_rn_call(double h) { return cube_rn(h); }

HC_DEV double icube_rn(double h) {
  const unsigned long long H = (unsigned long long)__double_as_longlong(h);
  const int eh = (int)(H >> 52) & 0x7ff;
  // the cube's biased exponent is 3 eh - 2046 + k (k = 0..2) before
  // rounding: keep it within [1, 2045]
  if (eh < 683 || eh > 1363) return cube_rn_call(h);
  const unsigned long long M52 = (1ull << 52) - 1;
  const unsigned long long m = (H & M52) | (1ull << 52);
  const unsigned long long a0 = m * m, a1 = __umul64hi(m, m);  // m^2 < 2^106
  const unsigned long long t0 = a0 * m, t1 = __umul64hi(a0, m);
  const unsigned long long u0 = a1 * m, u1 = __umul64hi(a1, m);
  const unsigned long long w1 = t1 + u0;
  const unsigned long long w2 = u1 + (w1 < t1 ? 1ull : 0ull);  // m^3 = w2:w1:t0, w2 < 2^31
  // top bit of m^3 at 156 + k
  const int k = (w2 >> 30) ? 2 : ((w2 >> 29) ? 1 : 0);
  const int sh = 104 + k;               // significand = m^3 >> sh (53 bits)
  const int r1 = sh - 64;               // 40..42: the shift within w2:w1
  unsigned long long sig = (w2 << (64 - r1)) | (w1 >> r1);
  const bool rbit = (w1 >> (r1 - 1)) & 1ull;
  const bool sticky = (w1 & ((1ull << (r1 - 1)) - 1)) != 0 || t0 != 0;
  int er = sh + 3 * (eh - 1075) + 1075;
  if (rbit && (sticky || (sig & 1ull))) sig++;
  if (sig == (1ull << 53)) {
    sig >>= 1;
    er++;
  }
  const unsigned long long sgn = H & 0x8000000000000000ull;
  return __longlong_as_double((long long)(sgn | ((unsigned long long)er << 52) | (sig & M52)));
}

// sqrt(x) rounded to nearest, on the integer pipe, for positive normal x:
// x = m' 2^E' with E' even and m' in [2^52, 2^54); s = floor(sqrt(m' 2^52))
// (53 bits) from a 64-bit reciprocal square root of m' (a float rsqrt.approx
// estimate, then two Newton-Raphson steps y (3 - u y^2) / 2 in fixed point),
// settled by the exact remainder r = m' 2^52 - s^2 and rounded up when
// r > s (a square root never falls on a midpoint).  Other x take the
// hardware square root through a call (kept out of line so that its FP64
// instructions are not predicated into the caller).
static __device__ __noinline__ double sqrt_call(double x) { return sqrt(x); }

HC_DEV double isqrt_rn(double x) {
  const unsigned long long X = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)(X >> 52) & 0x7ff;
  if ((X >> 63) || ex == 0 || ex == 0x7ff) return sqrt_call(x);
  const unsigned long long m = (X & ((1ull << 52) - 1)) | (1ull << 52);
  const int E = ex - 1075;
  const int odd = E & 1;
  const unsigned long long mp = m << odd;  // [2^52, 2^54)
  const int big = (mp >> 53) ? 1 : 0;
  const float uf =
      __uint_as_float((unsigned)((127 + big) << 23) | (unsigned)((mp >> (29 + big)) & 0x7fffffu));
  float r0;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(uf));
  const unsigned rb = __float_as_uint(r0);  // r0 in (0.5, 1]
  unsigned long long Y = (unsigned long long)((rb & 0x7fffffu) | 0x800000u) << ((int)(rb >> 23) - 87);
#pragma unroll
  for (int k = 0; k < 2; k++) {  // Y ~ 2^63 / sqrt(m' / 2^52)
    const unsigned long long P_hi = __umul64hi(Y, Y);
    const unsigned long long lo = mp * P_hi, hi = __umul64hi(mp, P_hi);
    const unsigned long long W = (hi << 12) | (lo >> 52);  // ~2^62 u y^2
    const long long E0 = (long long)((1ull << 62) - W);  // ~2^62 (1 - u y^2), small
    const unsigned long long aE = (E0 < 0) ? (unsigned long long)(-E0) : (unsigned long long)E0;
    const unsigned long long c = (__umul64hi(Y, aE) << 1) | ((Y * aE) >> 63);  // Y |E0| / 2^63
    Y = (E0 < 0) ? Y - c : Y + c;
  }
  unsigned long long s = (__umul64hi(mp, Y) << 1) | ((mp * Y) >> 63);
  long long r = (long long)((mp << 52) - s * s);  // exact: |r| < 2^63
  if (r < 0) {
    s--;
    r += (long long)(2 * s + 1);
  }
  if (r < 0) {
    s--;
    r += (long long)(2 * s + 1);
  }
  if (r > (long long)(2 * s)) {
    r -= (long long)(2 * s + 1);
    s++;
  }
  if (r > (long long)(2 * s)) {
    r -= (long long)(2 * s + 1);
    s++;
  }
  int er = (E - odd - 52) / 2 + 1075;
  if (r > (long long)s) s++;
  if (s == (1ull << 53)) {
    s >>= 1;
    er++;
  }
  return __longlong_as_double((long long)(((unsigned long long)er << 52) | (s & ((1ull << 52) - 1))));
}

// RN(a / b), the IEEE quotient, computed on the integer pipe.  On this GPU
// the FP64 pipe retires two lanes per clock per SM, an IEEE division takes
// about nine of its instructions, and a warp's integer multiply-add costs a
// thirtieth of one FP64 instruction; the stencils are FP64-pipe bound.
//
// Significands ma (normalised so that mb <= ma < 2 mb) and mb (53 bits):
// the quotient's significand is q = floor(ma 2^52 / mb), exact remainder
// r = ma 2^52 - q mb, rounded up when 2r > mb (2r == mb cannot occur for a
// quotient of 53-bit significands, and is rounded to even regardless).
// q comes from a 64-bit reciprocal V of mb: a float estimate (rcp.approx,
// relative error below 2^-21 after truncating mb to 24 bits), then two
// Newton-Raphson steps x + x (1 - mb x) in fixed point, each of which stays
// below 2^116/mb; the second leaves V within two units of it, so
// floor(ma V / 2^64) is q or q - 1, and the remainder settles it.  A zero
// dividend gives the signed zero; other operands that are zero, subnormal,
// infinite or NaN, and quotients that would leave the normal range, take the
// hardware division.
//
// An hc_divisor holds the divisor's part (V), so quotients by one divisor
// share it: ddiv_prep(b) once, then ddiv_by(a, d) per dividend.  Divisors
// fixed for a run are prepared on the host (host_divisor, exact V).
HC_DEV hc_divisor ddiv_prep(double b) {
  const unsigned long long B = (unsigned long long)__double_as_longlong(b);
  const unsigned long long M52 = (1ull << 52) - 1, H52 = 1ull << 52;
  hc_divisor d;
  d.b = b;
  d.eb = (int)(B >> 52) & 0x7ff;
  d.ok = d.eb != 0 && d.eb != 0x7ff;
  const unsigned long long mb = (B & M52) | H52;
  d.mb = mb;
  d.V = 0;
  if (mb != H52) {
    // float estimate of 2^83/mb from the top 24 bits of mb, as an integer
    const float fm = __uint_as_float(0x3f800000u | (unsigned)((mb >> 29) & 0x7fffffu));
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(fm));
    const unsigned rb = __float_as_uint(rf);  // rf in (0.5, 1]
    const unsigned long long R0 = (unsigned long long)((rb & 0x7fffffu) | 0x800000u)
                                  << ((int)(rb >> 23) - 119);
    // Newton step at 2^83: E = 2^83 - mb R0, |E| < 2^62 (low 64 bits suffice)
    const long long E = (long long)(0ull - mb * R0);
    const unsigned long long plo = R0 * (unsigned long long)E;
    const unsigned long long phi = (unsigned long long)__mul64hi((long long)R0, E);
    unsigned long long V = (R0 << 33) + ((phi << 14) | (plo >> 50));  // ~2^116/mb
    // Newton step at 2^116: E2 = 2^116 - mb V in [0, 2^74), kept as E2 / 2^20
    const unsigned long long qlo = mb * V, qhi = __umul64hi(mb, V);
    const unsigned long long e_lo = 0ull - qlo;
    const unsigned long long e_hi = H52 - qhi - (qlo != 0 ? 1ull : 0ull);
    const unsigned long long e_s = (e_hi << 44) | (e_lo >> 20);
    d.V = V + (__umul64hi(V, e_s) >> 32);
  }
  return d;
}

// The hardware division, out of line: inlined, the compiler predicates its
// FP64 instructions into every call site, where they take FP64 issue slots
// whether the fallback runs or not.
static __device__ __noinline__ double ddiv_hw(double a, double b) { return __ddiv_rn(a, b); }

HC_DEV double ddiv_by(double a, const hc_divisor& d) {
  const unsigned long long A = (unsigned long long)__double_as_longlong(a);
  const unsigned long long M52 = (1ull << 52) - 1, H52 = 1ull << 52;
  const int ea = (int)(A >> 52) & 0x7ff;
  unsigned long long ma = (A & M52) | H52;
  const unsigned long long mb = d.mb;
  int er = ea - d.eb + 1023;
  if (ma < mb) {
    ma <<= 1;
    er--;
  }
  if (!d.ok || ea == 0 || ea == 0x7ff || er < 1 || er > 2045) {
    // a zero dividend (frequent: flat water surfaces, cells with no net
    // flux) gives the signed zero here rather than in the hardware division
    if (d.ok && (A << 1) == 0)
      return __longlong_as_double(
          (long long)((A ^ (unsigned long long)__double_as_longlong(d.b)) & 0x8000000000000000ull));
    return ddiv_hw(a, d.b);
  }
  unsigned long long q, r;
  if (mb == H52) {  // b a power of two: exact
    q = ma;
    r = 0;
  } else {
    q = __umul64hi(ma, d.V);
    r = (ma << 52) - q * mb;
    if (r >= mb) {
      r -= mb;
      q++;
    }
    if (r >= mb) {
      r -= mb;
      q++;
    }
  }
  const unsigned long long r2 = r << 1;
  if (r2 > mb || (r2 == mb && (q & 1))) q++;
  if (q == (H52 << 1)) {
    q = H52;
    er++;
  }
  const unsigned long long sgn = (A ^ (unsigned long long)__double_as_longlong(d.b)) &
                                 0x8000000000000000ull;
  return __longlong_as_double((long long)(sgn | ((unsigned long long)er << 52) | (q & M52)));
}

HC_DEV double ddiv_rn(double a, double b) { return ddiv_by(a, ddiv_prep(b)); }

// hc_divisor for a divisor fixed for the run, V exact (floor(2^116/mb))
hc_divisor host_divisor(double b);

// (double)f on the integer pipe for normal floats and zeros, the conversion
// instruction (an FP64-pipe operation) otherwise.
HC_DEV double f2d_i(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  if (ex == 0 || ex == 0xffu) {
    if ((u & 0x7fffffffu) == 0)
      return __longlong_as_double((long long)((unsigned long long)(u & 0x80000000u) << 32));
    return (double)f;
  }
  return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                          ((unsigned long long)(ex - 127 + 1023) << 52) |
                                          ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// (float)x, rounded to nearest-even, on the integer pipe for results in the
// float normal range and zeros, the conversion instruction otherwise.
HC_DEV float d2f_i(double x) {
  const unsigned long long X = (unsigned long long)__double_as_longlong(x);
  const unsigned sgn = (unsigned)(X >> 32) & 0x80000000u;
  const int ef = ((int)(X >> 52) & 0x7ff) - 1023 + 127;
  if (ef < 1 || ef > 253) {
    if ((X << 1) == 0) return __uint_as_float(sgn);
    return (float)x;
  }
  const unsigned long long mant = X & ((1ull << 52) - 1);
  unsigned m = (unsigned)(mant >> 29), e = (unsigned)ef;
  const unsigned long long rem = mant & ((1ull << 29) - 1), half = 1ull << 28;
  if (rem > half || (rem == half && (m & 1u))) {
    if (++m == (1u << 23)) {
      m = 0;
      e++;
    }
  }
  return __uint_as_float(sgn | (e << 23) | m);
}

// A float within a relative 2^-20 of |x| (or 0 / +inf when |x| is outside
// the float normal range), built with integer operations only: the FP64
// pipe is the scarce resource on this GPU, and these estimates only decide
// which side of a threshold a value lies on (see near_or_above).
HC_DEV float approx_abs_f(double x) {
  const int hi = __double2hiint(x);
  const int e = ((hi >> 20) & 0x7ff) - 1023 + 127;
  if (e <= 0) return 0.0f;
  if (e >= 255) return __int_as_float(0x7f800000);
  return __int_as_float((e << 23) | ((hi & 0xfffff) << 3));
}

// Signed variant of approx_abs_f.
HC_DEV float approx_f(double x) {
  const int hi = __double2hiint(x);
  const float a = approx_abs_f(x);
  return (hi < 0) ? -a : a;
}

// static_cast<int>(double) as the reference's x86-64 build executes it
// (cvttsd2si): NaN or out-of-range values give INT_MIN.
HC_DEV int x86_trunc_to_int(double v) {
  if (!(v > -2147483649.0 && v < 2147483648.0)) return (int)0x80000000u;
  return (int)v;
}

HC_DEV void atomic_max_pos(unsigned long long* a, double v) {
  // valid for v >= +0.0: the IEEE bit pattern orders like the value
  atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

// A cell's grain record lives in its own slot, its fractions side by side:
// the grain row (fractions 0..HC_G) in 12 doubles (96 bytes, three 32-byte
// sectors), the strata (10 layers x HC_ST_N fractions) in 90.  Every kernel
// reads and writes a record whole, and the cells it visits are gathered
// (wet lists, chains), so a record costs three sectors instead of one per
// fraction.
constexpr size_t kGrainStride = 12;
constexpr size_t kStrataStride = 10 * HC_ST_N;
HC_DEV double& grain_at(const hc_view& c, size_t cell, int n) {
  return c.grain[cell * kGrainStride + n];
}
HC_DEV double& strata_at(const hc_view& c, size_t cell, int z, int n) {
  return c.strata[cell * kStrataStride + (size_t)z * HC_ST_N + n];
}

// addGS :3949-3983 for a record held in the cell's own slot (the caller
// assigns the reference's row number).  sort_active on a fresh record is a
// no-op whenever dprop[1..9] sums to about 1; callers that need it run it.
HC_DEV void grain_record_init(const hc_view& c, size_t cell, double elev, double bedrock) {
  const hc_params& p = c.p;
  const double active = p.active;
  grain_at(c, cell, 0) = 0;
  for (int n = 1; n <= HC_G - 1; n++) grain_at(c, cell, n) = active * p.dprop[n];
  grain_at(c, cell, HC_G) = 0;
  for (int z = 0; z <= 9; z++) {
    bool below = elev - (active * (z + 1)) < (bedrock - active);
    for (int n2 = 0; n2 <= HC_G - 2; n2++)
      strata_at(c, cell, z, n2) = below ? 0.0 : (active)*p.dprop[n2 + 1];
  }
}

// launch helpers (defined in hc_api.cu)
hc_status hc_fail(hc_ctx* c, hc_status st, const char* fmt, ...);
hc_status hc_cuda(hc_ctx* c, cudaError_t e, const char* what);

// phases of one iteration (hc_flow.cu, hc_erode.cu, hc_slide.cu, hc_lateral.cu)
void launch_control(hc_ctx* c);          // scalar driver logic up to flow_route
                                         // (sets c->hcur's conditions when capturing)
void launch_inputs(hc_ctx* c);           // catchment input points
void launch_flow_dt(hc_ctx* c);          // flow_timestep for member-level calls
void launch_flow_route(hc_ctx* c, int gated);
void launch_depth_update(hc_ctx* c, int gated);
void launch_scan_area(hc_ctx* c, int gated);
void launch_wet_list(hc_ctx* c, int gated);  // rebuild the wet-cell list from the mask
void launch_flux_out(hc_ctx* c, int gated, int record);
// k_flow_route's launch shapes (hc_flow.cu) and the autotuner (hc_tune.cu)
struct FlowShape {
  int minb;     // blocks of 256 per multiprocessor (register budget)
  int waves;    // grid = SMs x minb x waves; 0: the wet-list default grid
  int compact;  // 1: the face-compacted kernel (k_flow_route_q); 2: the same
                // with its divisions through one out-of-line copy
};
constexpr int kFlowShapeCount = 18;
static_assert(kFlowShapeCount <= kMaxFlowShapes, "hc_ctx::tune_ms holds every shape");
extern const FlowShape kFlowShapes[kFlowShapeCount];
void launch_flow_route_shape(hc_ctx* c, int gated, int shape);
hc_status autotune(hc_ctx* c, bool force);
void launch_volume(hc_ctx* c);           // hc_dev::vol_now = depth sum of the grid
void launch_mass_reset(hc_ctx* c);       // the ledger starts again from vol_now
void launch_erode_begin(hc_ctx* c, int gated, double mult);
// next: the conditional handle of the following pass (set when retrying);
// has_next 0 outside graph capture
void launch_erode_pass(hc_ctx* c, int max_passes, cudaGraphConditionalHandle next = 0,
                       int has_next = 0);
void launch_erode_finish(hc_ctx* c, int gated);
void launch_lateral_check(hc_ctx* c);
size_t erode_scratch_bytes(size_t N2, int imax, int jmax);
void launch_slide3(hc_ctx* c, int gated);
hc_status run_lateral(hc_ctx* c);
hc_status run_global_landsliding(hc_ctx* c, int* sweeps);
hc_status run_creep(hc_ctx* c, double time);
size_t slide_scratch_bytes(size_t N2, int n);  // n = max(imax, jmax)

// host helpers (hc_host.cpp)
// the drainage sweep order (std::sort's permutation, exact); cached while
// the elevations are unchanged (*reused)
const uint32_t* host_drainage_order(const hc_params* p, const double* elev, void* cache,
                                    bool* reused);
// sort_order(c, el, order): the sweep order for the elevations el (device)
// into order (device, N2 entries)
hc_status run_drainage_device(hc_ctx* c, const double* el, bool area_valid,
                              hc_status (*sort_order)(hc_ctx*, const double*, uint32_t*),
                              bool* sorted);
// device sort (hc_sort.cu): std::sort's permutation of the drainage pairs
// (or of n values); *fallback when the host's exact sort must run instead
struct hc_sort_work* sort_work_new();
void sort_work_free(struct hc_sort_work* w);
cudaError_t device_drainage_order(hc_ctx* c, const double* el, uint32_t* order, bool* fallback);
cudaError_t device_sort_values(struct hc_sort_work* w, const double* v, size_t n, uint32_t* perm,
                               cudaStream_t s, bool* fallback, int64_t* launches);
void host_sort_exact(std::pair<double, double>* a, size_t n, int threads);
void launch_adj_save(hc_ctx* c);         // adjoint replay: state before the iteration
hc_status ctx_pull(hc_ctx* c);   // control block device -> host mirror
hc_status ctx_push(hc_ctx* c);   // host mirror -> device
const float* ctx_rain(hc_ctx* c, int* rows, int* cols);  // host copy of the rain table
hc_status hc_fail(hc_ctx* c, hc_status st, const char* fmt, ...);
hc_status hc_cuda(hc_ctx* c, cudaError_t e, const char* what);
void* host_drainage_cache_new();
void host_drainage_cache_free(void* p);
void host_topmodel_tangent(const hc_params* p, const float* rain, int rows, int cols, int nsteps,
                           double* d_old, double* d_new);
void host_topmodel_table(const hc_params* p, const float* rain, int rows, int cols,
                         int nsteps, double* table /* [nsteps][2][rfnum+1] */);
