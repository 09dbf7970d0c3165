// Slope failure and creep:
//   in_channel_landsliding :5429-5527 ("slide_3", every 10 iterations)
//   global_landsliding     :5529-5654 (daily; its serial sweep runs on a host
//                          core, hc_host.cpp)
//   creep                  :5293-5427 (host-driven, every 10 days)
//
// slide_3 and global landsliding are sequential relaxations: every test sees
// the elevations left by the moves before it, in the reference's loop order.
// Moves are rare (a drop steeper than the failure angle over one cell), so
// the device first tests every cell against the elevations at the start of
// the sweep, in parallel.  If no test passes, the serial sweep would move
// nothing either and the sweep is over.  Otherwise one thread replays the
// sweep in loop order, visiting only (a) the cells whose test passed and
// (b) cells later in the loop whose 3x3 neighbourhood a move has changed -
// every other cell would evaluate its tests on unchanged elevations, where
// they failed.  The result is the serial sweep's, move for move.

#include "hc_grain.cuh"

#include <math.h>
#include <climits>
#include <cmath>
#include <vector>

namespace {

// neighbour order of the eight tests (:5457-5522 and :5561-5641)
__constant__ int kSx[8] = {1, 0, -1, -1, -1, 0, 1, 1};
__constant__ int kSy[8] = {1, 1, 1, 0, -1, -1, -1, 0};

struct SlideScratch {
  uint8_t* flag;        // N2 bytes, one per loop position
  int32_t* list;        // positions whose test passed, in loop order
  int32_t* block_sums;
  int32_t* count;
  int32_t* heap;        // pending re-tests
  int heap_cap;
  double* total;        // global landsliding: sum of moves of the sweep
};

// Loop position of a cell.  slide_3 walks columns (y outer, the wet rows of
// down_scan inner); global landsliding walks rows (x outer, y inner).
struct Order {
  int col_major;  // 1: P = y*(imax+2) + x ; 0: P = x*(jmax+2) + y
  int imax, jmax;
  __device__ __forceinline__ long long pos(int x, int y) const {
    return col_major ? (long long)y * (imax + 2) + x : (long long)x * (jmax + 2) + y;
  }
  __device__ __forceinline__ void cell(long long P, int& x, int& y) const {
    if (col_major) {
      y = (int)(P / (imax + 2));
      x = (int)(P % (imax + 2));
    } else {
      x = (int)(P / (jmax + 2));
      y = (int)(P % (jmax + 2));
    }
  }
};

// The eight tests of one visit.  slide3: the cell is the clamped row of a
// down_scan entry, failure at tan(angle)*DX or 10000 when at the bedrock
// floor, moves go through slide_GS.  global: cap at ERODEFACTOR, floor factor
// 10*DX, no grain bookkeeping.  `probe`: test only, no moves.
__device__ bool slide_visit(const hc_view& c, hc_dev* d, int x, int y, double factor, bool global,
                            bool probe, double* total, int* moved_dirs) {
  const size_t W = c.W;
  const size_t cell = (size_t)x * W + y;
  const double active = c.p.active;
  double wet_factor = factor;
  if (c.elev[cell] <= (c.bed[cell] + active)) wet_factor = global ? 10 * c.p.DX : 10000;
  bool any = false;
  int moved = 0;
  for (int k = 0; k < 8; k++) {
    const int x2 = x + kSx[k], y2 = y + kSy[k];
    const size_t nb = (size_t)x2 * W + y2;
    const bool diag = (kSx[k] != 0 && kSy[k] != 0);
    const double e = c.elev[cell], e2 = c.elev[nb];
    const double drop = diag ? ((e - e2) / 1.41) : (e - e2);
    if (drop > wet_factor && e2 > -9999) {
      any = true;
      if (probe) return true;
      double diff = (diag ? ((e - e2) / 1.41) : (e - e2)) - wet_factor;
      if ((e - diff) < (c.bed[cell] + active)) diff = (e - (c.bed[cell] + active));
      if (global && diff > c.p.ERODEFACTOR) diff = c.p.ERODEFACTOR;
      c.elev[cell] = e - diff;
      c.elev[nb] = e2 + diff;
      if (global) *total += diff;
      else slide_GS_dev(c, d, cell, diff, nb, true);
      moved |= 1 << k;
    }
  }
  if (moved_dirs) *moved_dirs = moved;
  return any;
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

// The visit as the serial replay makes it: the eight neighbours' elevations
// are loaded together (one round trip instead of eight dependent ones), a
// diagonal test is first decided on a float estimate and its FP64 division
// evaluated only near the threshold, and moves update the held values.  The
// tests, moves and their order are slide_visit's; returns the moved
// directions.
__device__ int slide_visit_held(const hc_view& c, hc_dev* d, int x, int y, double factor,
                                bool global, double* total) {
  constexpr int dxs[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  constexpr int dys[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  const size_t W = c.W;
  const size_t cell = (size_t)x * W + y;
  const double active = c.p.active;
  double en[8];
#pragma unroll
  for (int k = 0; k < 8; k++) en[k] = c.elev[(size_t)(x + dxs[k]) * W + (y + dys[k])];
  double e = c.elev[cell];
  const double floor_e = c.bed[cell] + active;
  double wet_factor = factor;
  if (e <= floor_e) wet_factor = global ? 10 * c.p.DX : 10000;
  const float wf = approx_f(wet_factor);
  int moved = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const bool diag = dxs[k] != 0 && dys[k] != 0;
    const double e2 = en[k];
    if (!(dkey(e2) > kNoDataKey)) continue;  // e2 > -9999
    double drop;
    if (diag) {
      const float est = approx_f(e - e2) * (1.0f / 1.41f);
      const float m = 1e-4f * (fabsf(est) + fabsf(wf));
      if (m >= 1e-34f && m < 1e30f && est - wf < -m) continue;  // surely not above
      drop = (e - e2) / 1.41;
    } else {
      drop = e - e2;
    }
    if (!dgt(drop, wet_factor)) continue;
    double diff = drop - wet_factor;
    if ((e - diff) < floor_e) diff = (e - floor_e);
    if (global && diff > c.p.ERODEFACTOR) diff = c.p.ERODEFACTOR;
    const size_t nb = (size_t)(x + dxs[k]) * W + (y + dys[k]);
    e = e - diff;
    en[k] = e2 + diff;
    c.elev[cell] = e;
    c.elev[nb] = en[k];
    if (global) {
      *total += diff;
    } else {
      replay_slide_GS(c, d, cell, diff, nb);
    }
    moved |= 1 << k;
  }
  return moved;
}

// Phase 1: flag every loop position whose visit would move something now.
__global__ void k_slide_probe(const hc_view c, const hc_dev* d, uint8_t* flag, int global,
                              double factor, int gated) {
  if (gated && !(d->it_active && d->rest_active && d->do_slide)) return;
  const int y = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (x > c.imax || y > c.jmax) return;
  const size_t cell = (size_t)x * c.W + y;
  uint8_t f = 0;
  if (global) {
    if (x >= 2 && x <= c.imax - 1 && y >= 2 && y <= c.jmax - 1)
      f = slide_visit(c, nullptr, x, y, factor, true, true, nullptr, nullptr) ? 1 : 0;
  } else if (y >= 2 && y <= c.jmax - 1 && c.mask[cell]) {
    int xc = x;
    if (xc == c.imax) xc = c.imax - 1;
    if (xc == 1) xc = 2;
    f = slide_visit(c, nullptr, xc, y, factor, false, true, nullptr, nullptr) ? 1 : 0;
  }
  // flags are indexed by loop position
  Order o{global ? 0 : 1, c.imax, c.jmax};
  flag[o.pos(x, y)] = f;
}

__global__ void k_flag_count(const uint8_t* flag, size_t n, int32_t* block_sums, const hc_dev* d,
                             int gated) {
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
}

__global__ void k_flag_scan(int32_t* block_sums, int nblocks, int32_t* total, const hc_dev* d,
                            int gated) {
  __shared__ int buf[1024];
  __shared__ int carry;
  if (gated && !(d->it_active && d->rest_active && d->do_slide)) return;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nblocks; base += 1024) {
    int k = base + threadIdx.x;
    int v = (k < nblocks) ? block_sums[k] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      int t = (threadIdx.x >= (unsigned)off) ? buf[threadIdx.x - off] : 0;
      __syncthreads();
      buf[threadIdx.x] += t;
      __syncthreads();
    }
    if (k < nblocks) block_sums[k] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
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
__device__ void heap_push(int32_t* h, int& n, int cap, int32_t v, hc_dev* d) {
  if (n >= cap) {
    d->err_code = 301;  // overflow: caught by the caller, which rescans
    return;
  }
  int i = n++;
  h[i] = v;
  while (i > 0) {
    int p = (i - 1) / 2;
    if (h[p] <= h[i]) break;
    int t = h[p];
    h[p] = h[i];
    h[i] = t;
    i = p;
  }
}
__device__ int32_t heap_pop(int32_t* h, int& n) {
  int32_t top = h[0];
  h[0] = h[--n];
  int i = 0;
  for (;;) {
    int l = 2 * i + 1, r = l + 1, m = i;
    if (l < n && h[l] < h[m]) m = l;
    if (r < n && h[r] < h[m]) m = r;
    if (m == i) break;
    int t = h[m];
    h[m] = h[i];
    h[i] = t;
    i = m;
  }
  return top;
}

// Queue the later loop positions whose visit reads a cell changed by the
// moves of a visit at (x, y): the visited cell and each moved-to neighbour
// (bit k of `moved`).  A visit reads the 3x3 block around its cell, so
// these are the positions whose cell lies within one of a changed cell;
// every other later position still sees the elevations the probe tested.
__device__ void push_affected(const hc_view& c, hc_dev* d, const Order& o, int x, int y, int moved,
                              long long Pcur, bool global, int32_t* heap, int& hn, int cap) {
  // cells of the 5x5 block around (x, y) within one of a changed cell
  unsigned need = 0;  // bit (dx+2)*5 + (dy+2)
  for (int k = -1; k < 8; k++) {
    if (k >= 0 && !((moved >> k) & 1)) continue;
    const int cx = (k < 0) ? 0 : kSx[k], cy = (k < 0) ? 0 : kSy[k];
    for (int dx = -1; dx <= 1; dx++)
      for (int dy = -1; dy <= 1; dy++) need |= 1u << ((cx + dx + 2) * 5 + (cy + dy + 2));
  }
  for (int dx = -2; dx <= 2; dx++)
    for (int dy = -2; dy <= 2; dy++) {
      if (!((need >> ((dx + 2) * 5 + (dy + 2))) & 1u)) continue;
      const int xx = x + dx, yy = y + dy;
      if (xx < 2 || xx > c.imax - 1 || yy < 2 || yy > c.jmax - 1) continue;
      if (global) {
        long long P = o.pos(xx, yy);
        if (P > Pcur) heap_push(heap, hn, cap, (int32_t)P, d);
      } else {
        // down_scan entries that visit row xx of column yy: xx itself, and the
        // clamped entries 1 -> 2 and imax -> imax-1
        const size_t W = c.W;
        if (c.mask[(size_t)xx * W + yy]) {
          long long P = o.pos(xx, yy);
          if (P > Pcur) heap_push(heap, hn, cap, (int32_t)P, d);
        }
        if (xx == 2 && c.mask[(size_t)1 * W + yy]) {
          long long P = o.pos(1, yy);
          if (P > Pcur) heap_push(heap, hn, cap, (int32_t)P, d);
        }
        if (xx == c.imax - 1 && c.mask[(size_t)c.imax * W + yy]) {
          long long P = o.pos(c.imax, yy);
          if (P > Pcur) heap_push(heap, hn, cap, (int32_t)P, d);
        }
      }
    }
}

__global__ void k_slide_replay(const hc_view c, hc_dev* d, const int32_t* list, const int32_t* count,
                               int32_t* heap, int heap_cap, int global, double factor,
                               double* total_out, int gated) {
  if (gated && !(d->it_active && d->rest_active && d->do_slide)) return;
  const int n = *count;
  if (total_out) *total_out = 0;
  if (n == 0) return;
  Order o{global ? 0 : 1, c.imax, c.jmax};
  int hn = 0, li = 0;
  long long last = -1;
  double total = 0;
  const int err0 = d->err_code;
  while (true) {
    long long cand = LLONG_MAX;
    if (li < n) cand = list[li];
    if (hn > 0 && heap[0] < cand) cand = heap[0];
    if (cand == LLONG_MAX) break;
    if (li < n && list[li] == cand) li++;
    while (hn > 0 && heap[0] <= cand) heap_pop(heap, hn);
    if (cand <= last) continue;
    last = cand;
    int x, y;
    o.cell(cand, x, y);
    int xc = x;
    if (!global) {
      if (xc == c.imax) xc = c.imax - 1;
      if (xc == 1) xc = 2;
    }
    const int moved = slide_visit_held(c, d, xc, y, factor, global != 0, &total);
    if (moved) push_affected(c, d, o, xc, y, moved, cand, global != 0, heap, hn, heap_cap);
    if (d->err_code == 301 && err0 != 301) {
      // heap overflow: finish the sweep visiting every later position
      d->err_code = err0;
      for (long long P = cand + 1;; P++) {
        int xx, yy;
        o.cell(P, xx, yy);
        if (global) {
          if (xx > c.imax - 1) break;
          if (yy < 2 || yy > c.jmax - 1 || xx < 2) continue;
          slide_visit_held(c, d, xx, yy, factor, true, &total);
        } else {
          if (yy > c.jmax - 1) break;
          if (xx < 1 || xx > c.imax || yy < 2) continue;
          if (!c.mask[(size_t)xx * c.W + yy]) continue;
          int x3 = xx;
          if (x3 == c.imax) x3 = c.imax - 1;
          if (x3 == 1) x3 = 2;
          slide_visit_held(c, d, x3, yy, factor, false, &total);
        }
      }
      break;
    }
  }
  d->s.grain_array_tot = d->grain_tot;
  if (total_out) *total_out = total;
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
  s.total = (double*)(base + off);
  off += 256;
  s.heap = (int32_t*)(base + off);
  s.heap_cap = 1 << 16;
  return s;
}

size_t slide_scratch_bytes(size_t N2) {
  size_t nblocks = (N2 + 1023) / 1024;
  return ((N2 + 255) / 256) * 256 + ((N2 * 4 + 255) / 256) * 256 + ((nblocks * 4 + 255) / 256) * 256 +
         512 + (size_t)(1 << 16) * 4 + 256;
}

static void slide_sweep(hc_ctx* c, int global, double factor, int gated) {
  SlideScratch s = slide_scratch(c);
  dim3 b(32, 8);
  dim3 g((c->v.jmax + b.x - 1) / b.x, (c->v.imax + b.y - 1) / b.y);
  // positions span the whole padded grid; unflagged positions must read 0
  cudaMemsetAsync(s.flag, 0, c->v.N2, c->cs);
  k_slide_probe<<<g, b, 0, c->cs>>>(c->v, c->dev, s.flag, global, factor, gated);
  count_launch(c, 1);
  const size_t n = c->v.N2;
  const int nblocks = (int)((n + 1023) / 1024);
  k_flag_count<<<nblocks, 1024, 0, c->cs>>>(s.flag, n, s.block_sums, c->dev, gated);
  count_launch(c, 1);
  k_flag_scan<<<1, 1024, 0, c->cs>>>(s.block_sums, nblocks, s.count, c->dev, gated);
  count_launch(c, 1);
  k_flag_compact<<<nblocks, 1024, 0, c->cs>>>(s.flag, n, s.block_sums, s.list, c->dev, gated);
  count_launch(c, 1);
  k_slide_replay<<<1, 1, 0, c->cs>>>(c->v, c->dev, s.list, s.count, s.heap, s.heap_cap, global,
                                    factor, s.total, gated);
  count_launch(c, 1);
}

static double slide_factor(const hc_ctx* c) {
  // std::tan((failureangle*(3.141592654/180)))*DX, evaluated on the host as
  // the reference does (libm tan)
  return std::tan((c->v.p.failureangle * (3.141592654 / 180))) * c->v.p.DX;
}

void launch_slide3(hc_ctx* c, int gated) { slide_sweep(c, 0, slide_factor(c), gated); }

hc_status run_global_landsliding(hc_ctx* c) {
  // a serial sweep over every cell, up to 200 times: one host core runs it
  // far faster than one GPU thread, and it touches elevations only
  const size_t N2 = c->v.N2;
  std::vector<double> elev(N2), bed(N2);
  cudaError_t e = cudaStreamSynchronize(c->s);
  if (e == cudaSuccess) e = cudaMemcpy(elev.data(), c->v.elev, N2 * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(bed.data(), c->v.bed, N2 * 8, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return hc_cuda(c, e, "global_landsliding");
  c->d2h_bytes += 2 * N2 * 8;
  host_global_landsliding(&c->v.p, bed.data(), elev.data());
  e = cudaMemcpy(c->v.elev, elev.data(), N2 * 8, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return hc_cuda(c, e, "global_landsliding");
  c->h2d_bytes += N2 * 8;
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
