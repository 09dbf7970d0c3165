// Slope failure and creep:
//   in_channel_landsliding :5429-5527 ("slide_3", every 10 iterations)
//   global_landsliding     :5529-5654 (daily: the same probe and warp replay
//                          over every cell, sweep after sweep, or a skewed
//                          wavefront when most cells move)
//   creep                  :5293-5427 (host-driven, every 10 days)
//
// slide_3 is a sequential relaxation: every test sees the elevations left by
// the moves before it, in the reference's loop order.  Moves are rare (a
// drop steeper than the failure angle over one cell), so the device first
// tests every cell against the elevations at the start of the sweep, in
// parallel.  If no test passes, the serial sweep would move nothing either
// and the sweep is over.  Otherwise one warp replays the sweep in loop
// order, visiting only (a) the cells whose test passed and (b) cells later
// in the loop whose 3x3 neighbourhood a move has changed - every other cell
// would evaluate its tests on unchanged elevations, where they failed.  The
// result is the serial sweep's, move for move.  Tests are decided on float
// estimates built with integer operations, and formed in FP64 only near the
// threshold: the FP64 pipe is this GPU's scarce unit.

#include "hc_grain.cuh"

#include <math.h>
#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

namespace {

struct SlideScratch {
  uint8_t* flag;        // N2 bytes, one per loop position
  int32_t* list;        // positions whose test passed, in loop order
  int32_t* block_sums;
  int32_t* count;
  uint32_t* ring;       // the replay's pending re-tests, when too many for shared memory
};

// The replay's pending re-tests: one bit per loop position in a ring of R
// positions, R the power of two >= 2*(imax+2) + 64.  A move at position P
// queues positions in (P, P + 2*(imax+2) + 4] only (the 5x5 block around its
// cell, columns y to y+2; +4 with the clamped rows 1 -> 2 and imax), so every
// pending position lies within R of the last one visited and has a bit of
// its own.
constexpr int kSharedRingWords = 8192;  // rings of up to 262,144 positions

__host__ __device__ inline int ring_words(int imax) {
  long long R = 64;
  while (R < 2LL * (imax + 2) + 64) R <<= 1;
  return (int)(R >> 5);
}

// Loop position of a cell: slide_3 walks columns (y outer, the wet rows of
// down_scan inner), P = y*(imax+2) + x.  Positions fit 32 bits, as the
// grid's cell count does.
struct Order {
  int H;  // imax + 2
  __device__ __forceinline__ int pos(int x, int y) const { return y * H + x; }
  __device__ __forceinline__ void cell(int P, int& x, int& y) const {
    y = P / H;
    x = P - y * H;
  }
};

// One test of a visit (:5457-5522): drop > w with drop = (e - e2)/1.41 on a
// diagonal, e - e2 otherwise.  Decided first on the estimates fe, fe2, fw of
// e, e2, w (approx_f: integer operations, within a relative 2^-20): the
// estimated drop is within 1.1 * 2^-20 * (|fe| + |fe2| + |fw|) (+ 2^-125
// for values below the float range) of (drop - w), and the margin m is eight
// times that.  Returns 0 when drop <= w surely, 1 when drop > w surely, 2
// when the FP64 test must decide (non-finite estimates give an infinite or
// NaN margin, and so 2).
__device__ __forceinline__ int drop_above_est(float fe, float fe2, float fw, bool diag) {
  float est = fe - fe2;
  if (diag) est *= (1.0f / 1.41f);
  const float m = 0x1p-17f * (fabsf(fe) + fabsf(fe2) + fabsf(fw)) + 1e-30f;
  const float t = est - fw;
  if (t < -m) return 0;
  if (t > m) return 1;
  return 2;
}

// the test in FP64, as the reference writes it (:5457-5522); out of line, so
// that the probe's eight call sites issue no FP64 work when they skip it
static __device__ __noinline__ bool drop_above_exact(double e, double e2, double w, bool diag) {
  const double drop = diag ? ((e - e2) / 1.41) : (e - e2);
  return drop > w && e2 > -9999;
}

// Whether the visit of the cell at (x, y) would move anything now.  Before a
// move all eight tests read the same elevations, so any passing test decides.
__device__ bool slide_probe_cell(const hc_view& c, int x, int y, double factor) {
  constexpr int dxs[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  constexpr int dys[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  const size_t W = c.W;
  const size_t cell = (size_t)x * W + y;
  double en[8];
#pragma unroll
  for (int k = 0; k < 8; k++) en[k] = c.elev[(size_t)(x + dxs[k]) * W + (y + dys[k])];
  const double e = c.elev[cell];
  const double wet_factor = (e <= (c.bed[cell] + c.p.active)) ? 10000.0 : factor;
  const float fe = approx_f(e), fw = approx_f(wet_factor);
  int undecided = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int r = drop_above_est(fe, approx_f(en[k]), fw, dxs[k] != 0 && dys[k] != 0);
    // r == 1: the estimates are finite, so the key compare is e2 > -9999
    if (r == 1 && dkey(en[k]) > kNoDataKey) return true;
    if (r == 2) undecided |= 1 << k;
  }
  if (!undecided) return false;
#pragma unroll
  for (int k = 0; k < 8; k++)
    if (((undecided >> k) & 1) && drop_above_exact(e, en[k], wet_factor, dxs[k] != 0 && dys[k] != 0))
      return true;
  return false;
}

// slide_GS for a move of the replay.  When both records exist, on the
// records held in registers (all loads issued together: the serial replay
// waits on latency); out of line, so that the eight tests of a visit share
// one copy of it.
static __device__ __noinline__ void replay_slide_GS(const hc_view& c, hc_dev* d, size_t cell,
                                                    double diff, size_t nb) {
  if (c.index[cell] != -9999 && c.index[nb] != -9999) {
    ApplyRow A, B;
    row_load(c, cell, 0, A);
    row_load(c, nb, 0, B);
    slide_GS_rows(c, d, cell, A, diff, nb, B, positive_total(A));
    row_store(c, cell, A);
    row_store(c, nb, B);
  } else {
    slide_GS_dev(c, d, cell, diff, nb, true);
  }
}

// The visit as the serial replay makes it (:5445-5525): the eight
// neighbours' elevations are loaded together (one round trip instead of
// eight dependent ones), each test is first decided on estimates
// (drop_above_est) and formed in FP64 only when it may pass, and moves update
// the held values.  The tests, moves and their order are the reference's;
// returns the moved directions (bit k: neighbour k).
__device__ int slide_visit_held(const hc_view& c, hc_dev* d, int x, int y, double factor) {
  constexpr int dxs[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  constexpr int dys[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  const size_t W = c.W;
  const size_t cell = (size_t)x * W + y;
  double en[8];
#pragma unroll
  for (int k = 0; k < 8; k++) en[k] = c.elev[(size_t)(x + dxs[k]) * W + (y + dys[k])];
  double e = c.elev[cell];
  const double floor_e = c.bed[cell] + c.p.active;
  const double wet_factor = (e <= floor_e) ? 10000.0 : factor;
  const float fw = approx_f(wet_factor);
  int moved = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const bool diag = dxs[k] != 0 && dys[k] != 0;
    const double e2 = en[k];
    if (drop_above_est(approx_f(e), approx_f(e2), fw, diag) == 0) continue;
    const double drop = diag ? ((e - e2) / 1.41) : (e - e2);
    if (!(drop > wet_factor && e2 > -9999)) continue;
    double diff = drop - wet_factor;
    if ((e - diff) < floor_e) diff = (e - floor_e);
    const size_t nb = (size_t)(x + dxs[k]) * W + (y + dys[k]);
    e = e - diff;
    en[k] = e2 + diff;
    c.elev[cell] = e;
    c.elev[nb] = en[k];
    replay_slide_GS(c, d, cell, diff, nb);
    moved |= 1 << k;
  }
  return moved;
}

// Phase 1: flag every loop position whose visit would move something now.
// Positions follow down_scan's rows, whose first and last wet rows visit the
// clamped rows 2 and imax-1 (:5436-5440).
__global__ void k_slide_probe(const hc_view c, const hc_dev* d, uint8_t* flag, double factor,
                              int gated) {
  if (gated && !(d->it_active && d->rest_active && d->do_slide)) return;
  const int y = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (x > c.imax || y > c.jmax) return;
  uint8_t f = 0;
  if (y >= 2 && y <= c.jmax - 1 && c.mask[(size_t)x * c.W + y]) {
    int xc = x;
    if (xc == c.imax) xc = c.imax - 1;
    if (xc == 1) xc = 2;
    f = slide_probe_cell(c, xc, y, factor) ? 1 : 0;
  }
  const Order o{c.imax + 2};
  flag[o.pos(x, y)] = f;
}

// Per-block counts of the flags; the block that finishes last scans them
// (exclusive, in place) and stores the total.
__global__ void __launch_bounds__(1024) k_flag_count(const uint8_t* flag, size_t n,
                                                     int32_t* block_sums, int32_t* total,
                                                     hc_dev* d, int gated) {
  __shared__ int ws[32];
  if (gated && !(d->it_active && d->rest_active && d->do_slide)) return;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int v = (i < n) ? flag[i] : 0;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < (int)blockDim.x / 32; k++) s += ws[k];
    block_sums[blockIdx.x] = s;
  }
  if (!last_to_arrive(&d->flag_arrive)) return;
  const int t = scan_block_counts(block_sums, (int)gridDim.x);
  if (threadIdx.x == 0) *total = t;
}

__global__ void k_flag_compact(const uint8_t* flag, size_t n, const int32_t* block_sums,
                               int32_t* list, const hc_dev* d, int gated) {
  __shared__ int ws[32];
  __shared__ int wb[32];
  if (gated && !(d->it_active && d->rest_active && d->do_slide)) return;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int v = (i < n) ? flag[i] : 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < (int)blockDim.x / 32; k++) {
      wb[k] = s;
      s += ws[k];
    }
  }
  __syncthreads();
  if (v) list[block_sums[blockIdx.x] + wb[warp] + incl - 1] = (int32_t)i;
}

// ---- the serial replay -----------------------------------------------------
// Queue the later loop positions whose visit reads a cell changed by the
// moves of a visit at (x, y): the visited cell and each moved-to neighbour
// (bit k of `moved`).  A visit reads the 3x3 block around its cell, so
// these are the positions whose cell lies within one of a changed cell;
// every other later position still sees the elevations the probe tested.
// The down_scan entries that visit row xx of column yy are xx itself and
// the clamped entries 1 -> 2 and imax -> imax-1.  Returns the number of
// positions newly set in the ring.
__device__ int push_affected(const hc_view& c, const Order& o, int x, int y, int moved, int Pcur,
                             uint32_t* ring, int RW) {
  constexpr int dxs[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  constexpr int dys[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  // cells of the 5x5 block around (x, y) within one of a changed cell:
  // bit (dx+2)*5 + (dy+2)
  unsigned need = 0;
#pragma unroll
  for (int k = -1; k < 8; k++) {
    if (k >= 0 && !((moved >> k) & 1)) continue;
    const int cx = (k < 0) ? 0 : dxs[k], cy = (k < 0) ? 0 : dys[k];
#pragma unroll
    for (int dx = -1; dx <= 1; dx++)
#pragma unroll
      for (int dy = -1; dy <= 1; dy++) need |= 1u << ((cx + dx + 2) * 5 + (cy + dy + 2));
  }
  // x and y lie in [2, imax-1] x [2, jmax-1], so every byte below is inside
  // the padded grid: all 35 are loaded together, before any test
  const size_t W = c.W;
  uint8_t mk[25], mt[5], mb[5];
#pragma unroll
  for (int b = 0; b < 25; b++) mk[b] = c.mask[(size_t)(x + b / 5 - 2) * W + (y + b % 5 - 2)];
#pragma unroll
  for (int j = 0; j < 5; j++) {
    mt[j] = c.mask[W + (y + j - 2)];
    mb[j] = c.mask[(size_t)c.imax * W + (y + j - 2)];
  }
  int added = 0;
  auto push = [&](int P) {
    if (P <= Pcur) return;
    uint32_t& w = ring[(P >> 5) & (RW - 1)];
    const uint32_t bit = 1u << (P & 31);
    if (!(w & bit)) {
      w |= bit;
      added++;
    }
  };
#pragma unroll
  for (int b = 0; b < 25; b++) {
    const int xx = x + b / 5 - 2, yy = y + b % 5 - 2;
    if (!((need >> b) & 1u) || xx < 2 || xx > c.imax - 1 || yy < 2 || yy > c.jmax - 1) continue;
    if (mk[b]) push(o.pos(xx, yy));
    if (xx == 2 && mt[b % 5]) push(o.pos(1, yy));
    if (xx == c.imax - 1 && mb[b % 5]) push(o.pos(c.imax, yy));
  }
  return added;
}

// The serial sweep in loop order over the flagged positions and the queued
// re-tests, by one warp.  A visit that moves nothing changes nothing, so the
// next kReplayBatch candidates in loop order are probed together, one per
// lane, against the current elevations; the candidates before the first one
// that moves are done, that one is visited in full by lane 0 (its moves
// depend on the moves before it), and the candidates after it stay queued,
// to be probed again on the changed elevations.  The visits and moves are
// the serial sweep's, in its order.
constexpr int kReplayBatch = 8;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ void replay_cell(const hc_view& c, const Order& o, int P, int& x,
                                            int& y) {
  o.cell(P, x, y);
  if (x == c.imax) x = c.imax - 1;  // the clamped first and last rows
  if (x == 1) x = 2;
}

__global__ void __launch_bounds__(32) k_slide_replay(const hc_view c, hc_dev* d,
                                                     const int32_t* list, const int32_t* count,
                                                     uint32_t* gring, double factor, int gated) {
  __shared__ uint32_t sring[kSharedRingWords];
  __shared__ int32_t batch[kReplayBatch];
  if (gated && !(d->it_active && d->rest_active && d->do_slide)) return;
  const int n = *count;
  if (n == 0) return;
  const int lane = threadIdx.x;
  const Order o{c.imax + 2};
  const int RW = ring_words(c.imax);
  const int R = RW << 5;
  uint32_t* ring = (RW <= kSharedRingWords) ? sring : gring;
  for (int i = lane; i < RW; i += 32) ring[i] = 0;
  __syncwarp();
  // the same on every lane: next list entry, last position visited, number
  // of positions pending in the ring
  int li = 0, last = -1, pend = 0;
  while (true) {
    const int L = (li < n) ? list[li] : INT_MAX;
    // the first pending positions of (last, min(L, last + R)), in order
    int nb = 0;
    if (pend > 0) {
      const int s0 = last + 1;
      const int end = (int)min((long long)L, (long long)last + R);
      for (int base = s0 & ~31; base < end && nb < kReplayBatch; base += 1024) {
        const int w0 = base + lane * 32;
        uint32_t bits = 0;
        if (w0 < end) {
          bits = ring[(w0 >> 5) & (RW - 1)];
          if (w0 < s0) bits &= ~0u << (s0 - w0);
          if (end - w0 < 32) bits &= (1u << (end - w0)) - 1u;
        }
        const int cnt = __popc(bits);
        int incl = cnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const int t = __shfl_up_sync(kFull, incl, off);
          if (lane >= off) incl += t;
        }
        int slot = nb + incl - cnt;
        while (bits && slot < kReplayBatch) {
          batch[slot++] = w0 + __ffs(bits) - 1;
          bits &= bits - 1;
        }
        nb = min(kReplayBatch, nb + __shfl_sync(kFull, incl, 31));
      }
    }
    const bool tookL = nb < kReplayBatch && L != INT_MAX;
    if (tookL) {
      if (lane == 0) batch[nb] = L;
      nb++;
    }
    if (nb == 0) break;
    __syncwarp();
    bool mv = false;
    if (lane < nb) {
      int x, y;
      replay_cell(c, o, batch[lane], x, y);
      mv = slide_probe_cell(c, x, y, factor);
    }
    const unsigned ball = __ballot_sync(kFull, mv);
    // candidates 0..upto are visited now: before the first that moves, that
    // one, or all of them
    const int upto = ball ? (__ffs(ball) - 1) : nb - 1;
    int cleared = 0;
    if (lane <= upto) {
      const int P = batch[lane];
      const uint32_t bit = 1u << (P & 31);
      cleared = (atomicAnd(&ring[(P >> 5) & (RW - 1)], ~bit) & bit) ? 1 : 0;
    }
    pend -= __popc(__ballot_sync(kFull, cleared));
    if (tookL && upto == nb - 1) li++;
    last = batch[upto];
    if (ball) {
      int added = 0;
      if (lane == 0) {
        int x, y;
        replay_cell(c, o, last, x, y);
        const int moved = slide_visit_held(c, d, x, y, factor);
        if (moved) added = push_affected(c, o, x, y, moved, last, ring, RW);
      }
      pend += __shfl_sync(kFull, added, 0);
    }
    // lane 0's moves and pushes are visible to the warp's next turn
    __syncwarp();
  }
  if (lane == 0) d->s.grain_array_tot = d->grain_tot;
}

// ---- global_landsliding :5529-5654 ----------------------------------------
// The daily sweep visits every cell of rows 2..imax-1, columns 2..jmax-1,
// rows outer (cell order, so a loop position is the cell index), with the
// same eight tests in the same order as slide_3 but on elevations only
// (no grain records), the wet factor 10*DX below bedrock + active, and every
// move capped at ERODEFACTOR.  Sweeps repeat while the last one moved a
// positive total (at most 200).  As for slide_3: a parallel probe of every
// cell against the elevations at the start of the sweep, then one warp
// replays the sweep over the flagged cells and the later cells whose 3x3
// block a move changed.

struct GOrder {
  int W;  // jmax + 2
  __device__ __forceinline__ int pos(int x, int y) const { return x * W + y; }
  __device__ __forceinline__ void cell(int P, int& x, int& y) const {
    x = P / W;
    y = P - x * W;
  }
};

__device__ bool gslide_probe_cell(const hc_view& c, int x, int y, double factor) {
  constexpr int dxs[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  constexpr int dys[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  const size_t W = c.W;
  const size_t cell = (size_t)x * W + y;
  double en[8];
#pragma unroll
  for (int k = 0; k < 8; k++) en[k] = c.elev[(size_t)(x + dxs[k]) * W + (y + dys[k])];
  const double e = c.elev[cell];
  const double wet_factor = (e <= (c.bed[cell] + c.p.active)) ? 10 * c.p.DX : factor;
  const float fe = approx_f(e), fw = approx_f(wet_factor);
  int undecided = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int r = drop_above_est(fe, approx_f(en[k]), fw, dxs[k] != 0 && dys[k] != 0);
    if (r == 1 && dkey(en[k]) > kNoDataKey) return true;
    if (r == 2) undecided |= 1 << k;
  }
  if (!undecided) return false;
#pragma unroll
  for (int k = 0; k < 8; k++)
    if (((undecided >> k) & 1) && drop_above_exact(e, en[k], wet_factor, dxs[k] != 0 && dys[k] != 0))
      return true;
  return false;
}

// The visit (:5553-5630): the eight tests in order on the elevations held
// in registers, each move as the reference makes it; returns the moved
// directions and adds the moves to *total in order.
__device__ int gslide_visit(const hc_view& c, int x, int y, double factor, double* total) {
  constexpr int dxs[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  constexpr int dys[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  const size_t W = c.W;
  const size_t cell = (size_t)x * W + y;
  double en[8];
#pragma unroll
  for (int k = 0; k < 8; k++) en[k] = c.elev[(size_t)(x + dxs[k]) * W + (y + dys[k])];
  double e = c.elev[cell];
  const double bed = c.bed[cell], active = c.p.active, EF = c.p.ERODEFACTOR;
  double wet_factor = factor;
  if (e <= (bed + active)) wet_factor = 10 * c.p.DX;
  const float fw = approx_f(wet_factor);
  int moved = 0;
  for (int k = 0; k < 8; k++) {
    const bool diag = dxs[k] != 0 && dys[k] != 0;
    const double e2 = en[k];
    if (drop_above_est(approx_f(e), approx_f(e2), fw, diag) == 0) continue;
    const double drop = diag ? ((e - e2) / 1.41) : (e - e2);
    if (!(drop > wet_factor && e2 > -9999)) continue;
    double diff = drop - wet_factor;
    if ((e - diff) < (bed + active)) diff = (e - (bed + active));
    if (diff > EF) diff = EF;
    e -= diff;
    en[k] = e2 + diff;
    c.elev[cell] = e;
    c.elev[(size_t)(x + dxs[k]) * W + (y + dys[k])] = en[k];
    *total += diff;
    moved |= 1 << k;
  }
  return moved;
}

__global__ void k_gslide_probe(const hc_view c, uint8_t* flag, double factor) {
  const int y = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (x > c.imax || y > c.jmax) return;
  uint8_t f = 0;
  if (x >= 2 && x <= c.imax - 1 && y >= 2 && y <= c.jmax - 1)
    f = gslide_probe_cell(c, x, y, factor) ? 1 : 0;
  flag[(size_t)x * c.W + y] = f;
}

// The later positions whose visit reads a cell the visit at (x, y) changed
// (the cell and each moved-to neighbour): every cell of the loop within one
// of a changed cell.  All lie within 2*W + 2 positions of (x, y).
__device__ int gpush_affected(const hc_view& c, const GOrder& o, int x, int y, int moved, int Pcur,
                              uint32_t* ring, int RW) {
  constexpr int dxs[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  constexpr int dys[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  unsigned need = 0;
#pragma unroll
  for (int k = -1; k < 8; k++) {
    if (k >= 0 && !((moved >> k) & 1)) continue;
    const int cx = (k < 0) ? 0 : dxs[k], cy = (k < 0) ? 0 : dys[k];
#pragma unroll
    for (int dx = -1; dx <= 1; dx++)
#pragma unroll
      for (int dy = -1; dy <= 1; dy++) need |= 1u << ((cx + dx + 2) * 5 + (cy + dy + 2));
  }
  int added = 0;
  for (int b = 0; b < 25; b++) {
    const int xx = x + b / 5 - 2, yy = y + b % 5 - 2;
    if (!((need >> b) & 1u) || xx < 2 || xx > c.imax - 1 || yy < 2 || yy > c.jmax - 1) continue;
    const int P = o.pos(xx, yy);
    if (P <= Pcur) continue;
    uint32_t& w = ring[(P >> 5) & (RW - 1)];
    const uint32_t bit = 1u << (P & 31);
    if (!(w & bit)) {
      w |= bit;
      added++;
    }
  }
  return added;
}

// One sweep's replay by one warp, as k_slide_replay does it for slide_3;
// *total receives the sweep's total (the moves' sum in the serial order).
__global__ void __launch_bounds__(32) k_gslide_replay(const hc_view c, const int32_t* list,
                                                      const int32_t* count, uint32_t* gring,
                                                      double factor, double* total) {
  __shared__ uint32_t sring[kSharedRingWords];
  __shared__ int32_t batch[kReplayBatch];
  const int n = *count;
  const int lane = threadIdx.x;
  double tot = 0;
  if (n > 0) {
    const GOrder o{(int)c.W};
    const int RW = ring_words(c.jmax);
    const int R = RW << 5;
    uint32_t* ring = (RW <= kSharedRingWords) ? sring : gring;
    for (int i = lane; i < RW; i += 32) ring[i] = 0;
    __syncwarp();
    int li = 0, last = -1, pend = 0;
    while (true) {
      const int L = (li < n) ? list[li] : INT_MAX;
      int nb = 0;
      if (pend > 0) {
        const int s0 = last + 1;
        const int end = (int)min((long long)L, (long long)last + R);
        for (int base = s0 & ~31; base < end && nb < kReplayBatch; base += 1024) {
          const int w0 = base + lane * 32;
          uint32_t bits = 0;
          if (w0 < end) {
            bits = ring[(w0 >> 5) & (RW - 1)];
            if (w0 < s0) bits &= ~0u << (s0 - w0);
            if (end - w0 < 32) bits &= (1u << (end - w0)) - 1u;
          }
          const int cnt = __popc(bits);
          int incl = cnt;
#pragma unroll
          for (int off = 1; off < 32; off <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, off);
            if (lane >= off) incl += t;
          }
          int slot = nb + incl - cnt;
          while (bits && slot < kReplayBatch) {
            batch[slot++] = w0 + __ffs(bits) - 1;
            bits &= bits - 1;
          }
          nb = min(kReplayBatch, nb + __shfl_sync(kFull, incl, 31));
        }
      }
      const bool tookL = nb < kReplayBatch && L != INT_MAX;
      if (tookL) {
        if (lane == 0) batch[nb] = L;
        nb++;
      }
      if (nb == 0) break;
      __syncwarp();
      bool mv = false;
      if (lane < nb) {
        int x, y;
        o.cell(batch[lane], x, y);
        mv = gslide_probe_cell(c, x, y, factor);
      }
      const unsigned ball = __ballot_sync(kFull, mv);
      const int upto = ball ? (__ffs(ball) - 1) : nb - 1;
      int cleared = 0;
      if (lane <= upto) {
        const int P = batch[lane];
        const uint32_t bit = 1u << (P & 31);
        cleared = (atomicAnd(&ring[(P >> 5) & (RW - 1)], ~bit) & bit) ? 1 : 0;
      }
      pend -= __popc(__ballot_sync(kFull, cleared));
      if (tookL && upto == nb - 1) li++;
      last = batch[upto];
      if (ball) {
        int added = 0;
        if (lane == 0) {
          int x, y;
          o.cell(last, x, y);
          const int moved = gslide_visit(c, x, y, factor, &tot);
          if (moved) added = gpush_affected(c, o, x, y, moved, last, ring, RW);
        }
        pend += __shfl_sync(kFull, added, 0);
      }
      __syncwarp();
    }
  }
  if (lane == 0) *total = tot;
}

// A dense sweep (most cells move: a raw, unrelaxed DEM) as a skewed
// wavefront, one block: row r = x - 2 visits column y at step
// s = (y - 2) + 3 r.  A visit reads and writes only the 3x3 block around its
// cell, so two visits conflict only when their rows and their columns
// each differ by at most 2; every earlier visit that conflicts with the
// one at (x, y) (rows x-1 and x-2 up to column y+2, row x before y) runs at
// an earlier step, every later one at a later step, and visits of one step
// never conflict: the moves are the serial sweep's, in its order for every
// cell.  A thread takes rows r, r+1024, ...; the barrier between steps
// orders the global-memory writes.  *total: the sweep's moves summed per
// thread, then in thread order (the serial sum up to rounding; only its
// sign is used).
__global__ void __launch_bounds__(1024) k_gslide_wave(const hc_view c, double factor,
                                                      double* total) {
  const int rows = c.imax - 2, cols = c.jmax - 2;  // x in [2, imax-1], y in [2, jmax-1]
  double tot = 0;
  const int steps = (cols - 1) + 3 * (rows - 1) + 1;
  for (int st = 0; st < steps; st++) {
    for (int r = threadIdx.x; r < rows; r += blockDim.x) {
      const int y = 2 + st - 3 * r;
      if (y >= 2 && y <= c.jmax - 1) gslide_visit(c, r + 2, y, factor, &tot);
    }
    __syncthreads();
  }
  __shared__ double part[32];
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_down_sync(0xffffffffu, tot, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = tot;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) a += part[w];
    *total = a;
  }
}

// ---- creep :5293-5427 ------------------------------------------------------
// temp of the move from (x,y) to neighbour k, 0 when there is none
__device__ __forceinline__ double creep_temp(const hc_view& c, int x, int y, int k, double time) {
  const int cx[8] = {0, 1, 1, 1, 0, -1, -1, -1};
  const int cy[8] = {-1, -1, 0, 1, 1, 1, 0, -1};
  const size_t cell = (size_t)x * c.W + y;
  const double e = c.elev[cell], bed = c.bed[cell];
  if (!(e > bed)) return -1;  // no move (distinguished from a zero move)
  const size_t nb = (size_t)(x + cx[k]) * c.W + (y + cy[k]);
  const double e2 = c.elev[nb];
  if (!(e2 < e && e2 > -9999)) return -1;
  const bool diag = (cx[k] != 0 && cy[k] != 0);
  const double root = 7.07, DX = c.p.DX, CR = c.p.CREEP_RATE;
  double temp = diag ? ((e - e2) / root) * CR * time / root : ((e - e2) / DX) * CR * time / DX;
  if ((e - temp) < bed) temp = e - bed;
  if (temp < 0) temp = 0;
  return temp;
}

// tempcreep of each cell summed in the reference's order: moves are made by
// cells in row-major order, each cell its eight directions in turn.
__global__ void k_creep_gather(const hc_view c, double* tempcreep, double time) {
  const int y = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (x > c.imax || y > c.jmax) return;
  const int cx[8] = {0, 1, 1, 1, 0, -1, -1, -1};
  const int cy[8] = {-1, -1, 0, 1, 1, 1, 0, -1};
  double t = 0;
  auto src_ok = [&](int sx, int sy) { return sx >= 2 && sx <= c.imax - 1 && sy >= 2 && sy <= c.jmax - 1; };
  // sources before (x,y) in row-major order: (x-1, y-1), (x-1, y), (x-1, y+1), (x, y-1)
  const int before[4][2] = {{-1, -1}, {-1, 0}, {-1, 1}, {0, -1}};
  const int after[4][2] = {{0, 1}, {1, -1}, {1, 0}, {1, 1}};
  for (int b = 0; b < 4; b++) {
    const int sx = x + before[b][0], sy = y + before[b][1];
    if (!src_ok(sx, sy)) continue;
    for (int k = 0; k < 8; k++)
      if (sx + cx[k] == x && sy + cy[k] == y) {
        double v = creep_temp(c, sx, sy, k, time);
        if (v >= 0) t += v;
      }
  }
  if (src_ok(x, y))
    for (int k = 0; k < 8; k++) {
      double v = creep_temp(c, x, y, k, time);
      if (v >= 0) t -= v;
    }
  for (int b = 0; b < 4; b++) {
    const int sx = x + after[b][0], sy = y + after[b][1];
    if (!src_ok(sx, sy)) continue;
    for (int k = 0; k < 8; k++)
      if (sx + cx[k] == x && sy + cy[k] == y) {
        double v = creep_temp(c, sx, sy, k, time);
        if (v >= 0) t += v;
      }
  }
  tempcreep[(size_t)x * c.W + y] = t;
}

// grain transfers of creep, serial (only cells holding a grain record move
// grain, and a receiver may get its first record)
__global__ void k_creep_grain(const hc_view c, hc_dev* d, double time) {
  const int cx[8] = {0, 1, 1, 1, 0, -1, -1, -1};
  const int cy[8] = {-1, -1, 0, 1, 1, 1, 0, -1};
  for (int x = 2; x <= c.imax - 1; x++)
    for (int y = 2; y <= c.jmax - 1; y++) {
      const size_t cell = (size_t)x * c.W + y;
      if (c.index[cell] == -9999) continue;
      for (int k = 0; k < 8; k++) {
        double v = creep_temp(c, x, y, k, time);
        if (v >= 0) slide_GS_dev(c, d, cell, v, (size_t)(x + cx[k]) * c.W + (y + cy[k]), true);
      }
    }
  d->s.grain_array_tot = d->grain_tot;
}

__global__ void k_creep_apply(const hc_view c, const double* tempcreep) {
  const int y = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (x > c.imax || y > c.jmax) return;
  const size_t cell = (size_t)x * c.W + y;
  c.elev[cell] += tempcreep[cell];
}

__global__ void k_any_index(const hc_view c, int* any) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < c.N2 && c.index[i] != -9999) *any = 1;
}

}  // namespace

// ------------------------------------------------------------------ launches
static SlideScratch slide_scratch(hc_ctx* c) {
  SlideScratch s;
  char* base = (char*)c->v.touched;
  const size_t N2 = c->v.N2;
  s.flag = (uint8_t*)base;
  size_t off = ((N2 + 255) / 256) * 256;
  s.list = (int32_t*)(base + off);
  off += ((N2 * 4 + 255) / 256) * 256;
  size_t nblocks = (N2 + 1023) / 1024;
  s.block_sums = (int32_t*)(base + off);
  off += ((nblocks * 4 + 255) / 256) * 256;
  s.count = (int32_t*)(base + off);
  off += 256;
  s.ring = (uint32_t*)(base + off);
  return s;
}

// n: the longer side of the grid (slide_3's ring spans columns of imax+2
// positions, global landsliding's rows of jmax+2)
size_t slide_scratch_bytes(size_t N2, int n) {
  size_t nblocks = (N2 + 1023) / 1024;
  return ((N2 + 255) / 256) * 256 + ((N2 * 4 + 255) / 256) * 256 + ((nblocks * 4 + 255) / 256) * 256 +
         256 + (size_t)ring_words(n) * 4 + 256;
}

static void slide_sweep(hc_ctx* c, double factor, int gated) {
  SlideScratch s = slide_scratch(c);
  dim3 b(32, 8);
  dim3 g((c->v.jmax + b.x - 1) / b.x, (c->v.imax + b.y - 1) / b.y);
  // positions span the whole padded grid; unflagged positions must read 0
  cudaMemsetAsync(s.flag, 0, c->v.N2, c->cs);
  k_slide_probe<<<g, b, 0, c->cs>>>(c->v, c->dev, s.flag, factor, gated);
  count_launch(c, 1);
  const size_t n = c->v.N2;
  const int nblocks = (int)((n + 1023) / 1024);
  k_flag_count<<<nblocks, 1024, 0, c->cs>>>(s.flag, n, s.block_sums, s.count, c->dev, gated);
  count_launch(c, 1);
  k_flag_compact<<<nblocks, 1024, 0, c->cs>>>(s.flag, n, s.block_sums, s.list, c->dev, gated);
  count_launch(c, 1);
  k_slide_replay<<<1, 32, 0, c->cs>>>(c->v, c->dev, s.list, s.count, s.ring, factor, gated);
  count_launch(c, 1);
}

static double slide_factor(const hc_ctx* c) {
  // std::tan((failureangle*(3.141592654/180)))*DX, evaluated on the host as
  // the reference does (libm tan)
  return std::tan((c->v.p.failureangle * (3.141592654 / 180))) * c->v.p.DX;
}

void launch_slide3(hc_ctx* c, int gated) { slide_sweep(c, slide_factor(c), gated); }

// global_landsliding :5529-5654: sweeps while the last one moved a positive
// total, at most 200; each sweep a probe, the flagged cells' list and the
// replay, then one 16-byte read of the sweep's count and total.
hc_status run_global_landsliding(hc_ctx* c, int* sweeps) {
  SlideScratch s = slide_scratch(c);
  dim3 b(32, 8);
  dim3 g((c->v.jmax + b.x - 1) / b.x, (c->v.imax + b.y - 1) / b.y);
  const size_t n = c->v.N2;
  const int nblocks = (int)((n + 1023) / 1024);
  double* total = (double*)c->v.red;  // bytes 0-7 of the reduction scratch
  double h_total = 0;
  int32_t h_count = 0;
  int inc = 0;
  // More flagged cells than this: the wavefront (every cell, in about
  // jmax + 3 imax steps), else the replay of the flagged cells.
  const int dense = std::max(4096, (int)(c->v.imax + c->v.jmax));
  do {
    inc++;
    cudaMemsetAsync(s.flag, 0, n, c->s);
    k_gslide_probe<<<g, b, 0, c->s>>>(c->v, s.flag, slide_factor(c));
    k_flag_count<<<nblocks, 1024, 0, c->s>>>(s.flag, n, s.block_sums, s.count, c->dev, 0);
    count_launch(c, 2);
    cudaError_t e = cudaMemcpyAsync(&h_count, s.count, 4, cudaMemcpyDeviceToHost, c->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->s);
    if (e != cudaSuccess) return hc_cuda(c, e, "global_landsliding");
    if (h_count == 0) break;  // nothing moves: the sweep's total is 0
    if (h_count > dense) {
      k_gslide_wave<<<1, 1024, 0, c->s>>>(c->v, slide_factor(c), total);
      count_launch(c, 1);
    } else {
      k_flag_compact<<<nblocks, 1024, 0, c->s>>>(s.flag, n, s.block_sums, s.list, c->dev, 0);
      k_gslide_replay<<<1, 32, 0, c->s>>>(c->v, s.list, s.count, s.ring, slide_factor(c), total);
      count_launch(c, 2);
    }
    e = cudaMemcpyAsync(&h_total, total, 8, cudaMemcpyDeviceToHost, c->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->s);
    if (e != cudaSuccess) return hc_cuda(c, e, "global_landsliding");
    c->d2h_bytes += 12;
  } while (h_total > 0 && inc < 200);
  if (sweeps) *sweeps = inc;
  return HC_OK;
}

hc_status run_creep(hc_ctx* c, double time) {
  dim3 b(32, 8);
  dim3 g((c->v.jmax + b.x - 1) / b.x, (c->v.imax + b.y - 1) / b.y);
  double* tempcreep = c->v.erodetot;  // scratch field of N2 doubles
  k_creep_gather<<<g, b, 0, c->s>>>(c->v, tempcreep, time);
  count_launch(c, 1);
  int* any = (int*)((char*)c->v.red + 96);
  cudaMemsetAsync(any, 0, sizeof(int), c->s);
  k_any_index<<<(unsigned)((c->v.N2 + 255) / 256), 256, 0, c->s>>>(c->v, any);
  count_launch(c, 1);
  int h_any = 0;
  cudaError_t e = cudaMemcpyAsync(&h_any, any, sizeof(int), cudaMemcpyDeviceToHost, c->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->s);
  if (e != cudaSuccess) return hc_cuda(c, e, "creep");
  // grain transfers read the elevations before the creep is applied
  if (h_any) k_creep_grain<<<1, 1, 0, c->s>>>(c->v, c->dev, time);
  k_creep_apply<<<g, b, 0, c->s>>>(c->v, tempcreep);
  count_launch(c, 1);
  return HC_OK;
}
