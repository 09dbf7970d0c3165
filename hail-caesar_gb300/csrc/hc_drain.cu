// Drainage area and catchment input points, recomputed when the baseflow
// threshold moves (catchment_water_input_and_hydrology :3524-3539):
// zero_and_calc_drainage_area :2072-2089, drainage_area_D8 :2091-2271 and
// get_catchment_input_points :3741-3767.
//
// The reference sweeps all cells once from the highest to the lowest (an
// order fixed by a sort, hc_sort.cu) and pushes each cell's area to
// its lower neighbours.  A cell's final area is therefore its initial value
// plus the pushes of its higher neighbours, added in the order those were
// swept.  Here the same sums are pulled instead: a cell is ready once all
// its higher neighbours are done (Kahn's algorithm on the "higher than"
// graph), one frontier of ready cells per step, and each cell adds its
// neighbours' terms in their sweep order (the position in the sort, so equal
// elevations keep the reference's order).  Every term and every addition is
// the reference's, so the areas are bit-identical.  Cells the reference's
// loop never reaches (sorted position 0 and above imax*jmax, where the sort's
// padding pairs push them) keep area 0 and push nothing, as there.
//
// The sort itself is needed only where its order among equal elevations can
// show: two higher neighbours of one cell at the same elevation (the order
// of their pushes), or a group of equal elevations that straddles the first
// or the last reached position.  The device checks for those (a radix
// selection finds the last reached position); when none occurs, "reached" is
// a threshold on the elevation, the pushes are ordered by elevation, and no
// sort runs at all.  Otherwise the device sorts (hc_sort.cu; the host's
// exact sort where that declines).
//
// The elevations are those at the start of the iteration that moved the
// threshold (k_depth_update copies them before the iteration's erosion).

#include "hc_internal.cuh"

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <vector>

namespace {

__constant__ int kDrX[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1};
__constant__ int kDrY[9] = {0, -1, -1, 0, 1, 1, 1, 0, -1};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// unsigned key that orders like the elevations (std::sort's `<`: +0 == -0)
__host__ __device__ __forceinline__ unsigned long long ukey_bits(long long b) {
  const long long s = b >> 63;
  const long long k = ((b & 0x7fffffffffffffffLL) ^ s) - s;
  return (unsigned long long)k ^ 0x8000000000000000ULL;
}
__device__ __forceinline__ unsigned long long ukey(double x) {
  return ukey_bits(__double_as_longlong(x));
}
constexpr unsigned long long kZeroKey = 0x8000000000000000ULL;  // ukey(0.0)

__device__ __forceinline__ bool interior_ij(const hc_view& c, int& i, int& j) {
  j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  i = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  return i <= c.imax && j <= c.jmax;
}

// smallest elevation key
__global__ void k_drain_min(const hc_view c, const double* __restrict__ el) {
  int i, j;
  unsigned long long u = ~0ull;
  if (interior_ij(c, i, j)) u = ukey(el[(size_t)i * c.W + j]);
  for (int o = 16; o > 0; o >>= 1) u = min(u, __shfl_xor_sync(0xffffffffu, u, o));
  if ((threadIdx.x & 31) == 0) atomicMin(&c.drain_aux->min_u, u);
}

// how many cells share the smallest elevation, and whether any of them can
// receive area (an in-catchment cell, or a no-data cell below a neighbour)
__global__ void k_drain_mincount(const hc_view c, const double* __restrict__ el) {
  int i, j;
  if (!interior_ij(c, i, j)) return;
  const size_t W = c.W;
  const double e = el[(size_t)i * W + j];
  if (ukey(e) != c.drain_aux->min_u) return;
  atomicAdd(&c.drain_aux->min_count, 1u);
  bool matters = !(e == -9999);
  for (int dx = -1; dx <= 1; dx++)
    for (int dy = -1; dy <= 1; dy++) {
      const int i2 = i + dx, j2 = j + dy;
      if ((dx == 0 && dy == 0) || i2 < 1 || i2 > c.imax || j2 < 1 || j2 > c.jmax) continue;
      if (el[(size_t)i2 * W + j2] > e) matters = true;
    }
  if (matters) atomicOr(&c.drain_aux->min_matters, 1u);
}

// radix selection (8 bits a pass, most significant first) of the P-th
// largest key of the reference's sorted vector: the interior cells plus
// P = (imax+2)(jmax+2) - imax*jmax padding zeros
__global__ void k_sel_hist(const hc_view c, const double* __restrict__ el, int shift) {
  __shared__ unsigned int h[256];
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  const int nt = blockDim.x * blockDim.y;
  for (int k = t; k < 256; k += nt) h[k] = 0;
  __syncthreads();
  int i, j;
  const hc_drain_aux* a = c.drain_aux;
  if (interior_ij(c, i, j)) {
    const unsigned long long u = ukey(el[(size_t)i * c.W + j]);
    if ((u & a->mask) == a->prefix) atomicAdd(&h[(u >> shift) & 255], 1u);
  }
  __syncthreads();
  for (int k = t; k < 256; k += nt)
    if (h[k]) atomicAdd(&c.drain_aux->hist[k], h[k]);
}

__global__ void k_sel_pick(const hc_view c, int shift, unsigned long long padding) {
  hc_drain_aux* a = c.drain_aux;
  const unsigned long long zero_digit = (kZeroKey >> shift) & 255;
  const bool zero_in = (kZeroKey & a->mask) == a->prefix;
  unsigned long long cum = 0;
  int digit = 0;
  for (int d = 255; d >= 0; d--) {
    const unsigned long long n = a->hist[d] + ((zero_in && (unsigned)d == zero_digit) ? padding : 0);
    if (cum + n >= a->k) {
      digit = d;
      a->real_eq = a->hist[d];
      break;
    }
    cum += n;
  }
  a->k -= cum;
  a->gt += cum;
  a->prefix |= (unsigned long long)digit << shift;
  a->mask |= 255ull << shift;
  for (int d = 0; d < 256; d++) a->hist[d] = 0;
}

// sorted position of every cell the sweep reaches (1 .. imax*jmax); 0 = not
// reached
__global__ void k_drain_pos(const hc_view c, const uint32_t* __restrict__ order) {
  const size_t M = (size_t)c.imax * c.jmax;
  for (size_t n = 1 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; n <= M;
       n += (size_t)gridDim.x * blockDim.x) {
    const uint32_t cell = order[n];
    if (cell != 0) c.drain_pos[cell] = (uint32_t)n;
  }
}

// per interior cell: area = 0, the sum of downhill drops (difftot, the
// reference's clamped 8-neighbour loop in its order), the number of higher
// neighbours to wait for (cells with none start the first frontier), whether
// the sweep reaches the cell (drain_pos 1/0: below the selected last
// position, and not the unique lowest cell), and whether two higher
// neighbours share an elevation
__global__ void k_drain_init(const hc_view c, hc_dev* d, const double* __restrict__ el) {
  int i, j;
  if (!interior_ij(c, i, j)) return;
  const size_t W = c.W;
  const size_t cell = (size_t)i * W + j;
  const double e = el[cell];
  c.area[cell] = 0;
  double difftot = 0;
  for (int dir = 1; dir <= 8; dir++) {
    const int i2 = clampi(i + kDrX[dir], 1, c.imax), j2 = clampi(j + kDrY[dir], 1, c.jmax);
    const double e2 = el[(size_t)i2 * W + j2];
    if (dir % 2 != 0) {
      if (e2 < e) difftot += e - e2;
    } else {
      if (e2 < e) difftot += (e - e2) / 1.414;
    }
  }
  c.drain_dt[cell] = difftot;
  int higher = 0;
  double eh[8];
  bool tie = false;
  for (int dx = -1; dx <= 1; dx++)
    for (int dy = -1; dy <= 1; dy++) {
      const int i2 = i + dx, j2 = j + dy;
      if ((dx == 0 && dy == 0) || i2 < 1 || i2 > c.imax || j2 < 1 || j2 > c.jmax) continue;
      const double e2 = el[(size_t)i2 * W + j2];
      if (e2 > e) {
        for (int k = 0; k < higher; k++) tie |= (eh[k] == e2);
        eh[higher++] = e2;
      }
    }
  c.drain_pend[cell] = higher;
  if (tie) atomicOr(&c.drain_aux->contrib_tie, 1u);
  const hc_drain_aux* a = c.drain_aux;
  const unsigned long long u = ukey(e);
  const bool reached = !(u > a->prefix) &&
                       !(a->min_u < kZeroKey && a->min_count == 1 && u == a->min_u);
  c.drain_pos[cell] = reached ? 1u : 0u;
  if (higher == 0) {
    const unsigned k = atomicAdd(&d->drain_front, 1u);
    c.drain_f0[k] = (uint32_t)cell;
  }
}

// The share of each higher neighbour's area that reaches this cell, before
// the sweep: the reference's term (e_q - e)/difftot_q, or its diagonal form
// ((e_q - e)/1.414)/difftot_q, for the first direction of q whose (clamped)
// step lands here; neighbours with more than one such direction (at the
// edges) are marked and summed term by term in the sweep.  The sweep then
// adds aq * share, the reference's operations on the same values, and its
// critical path has no division (about 600 cycles each on this GPU's FP64
// pipe, against 128 for a multiply and an add).
__global__ void k_drain_frac(const hc_view c, const double* __restrict__ el) {
  int i, j;
  if (!interior_ij(c, i, j)) return;
  const size_t W = c.W, N2 = c.N2;
  const size_t cell = (size_t)i * W + j;
  const double e = el[cell];
  unsigned multi = 0;
  for (int kk = 0; kk < 9; kk++) {
    double g = 0;
    const int iq = i + kk / 3 - 1, jq = j + kk % 3 - 1;
    if (kk != 4 && iq >= 1 && iq <= c.imax && jq >= 1 && jq <= c.jmax) {
      const size_t q = (size_t)iq * W + jq;
      const double eq = el[q];
      if (eq > e) {
        const double dq = c.drain_dt[q];
        int found = 0;
        for (int dir = 1; dir <= 8; dir++) {
          const int i3 = clampi(iq + kDrX[dir], 1, c.imax), j3 = clampi(jq + kDrY[dir], 1, c.jmax);
          if (i3 != i || j3 != j) continue;
          if (found == 0) g = (dir % 2 != 0) ? ((eq - e) / dq) : (((eq - e) / 1.414) / dq);
          found++;
        }
        if (found > 1) multi |= 1u << kk;
      }
    }
    c.drain_frac[(size_t)kk * N2 + cell] = g;
  }
  c.drain_multi[cell] = (uint16_t)multi;
}

// Grid-wide barrier for k_drain_sweep, which is launched cooperatively (all
// blocks resident).  Sense by generation count; every wait is bounded: a
// block that gives up raises err and the sweep ends with an error status.
struct DrainSync {
  unsigned int arrive;
  unsigned int gen;
  unsigned int err;
  unsigned int count[3];  // frontier lengths, rotating by level
  unsigned int solo_level;            // level at which block 0 left its last solo run
  unsigned int pad;
  unsigned long long solo_done;       // cells done by then
};

// Frontiers of at most this many cells are swept by block 0 alone, level
// after level with block barriers, while the other blocks wait: most
// frontiers of a catchment hold a few hundred cells, and a grid barrier per
// level costs more than the work.
constexpr unsigned kSoloMax = 2048;

// `limit`: spins before giving up; `expect`: arrivals that open it (the
// number of blocks, unless a test asks for more)
__device__ __forceinline__ bool grid_barrier(DrainSync* g, unsigned expect, long limit) {
  __shared__ bool ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = true;
    const unsigned my = *(volatile unsigned*)&g->gen;
    __threadfence();
    if (atomicAdd(&g->arrive, 1u) == expect - 1) {
      g->arrive = 0;
      __threadfence();
      atomicAdd(&g->gen, 1u);
    } else {
      long spins = 0;
      while (*(volatile unsigned*)&g->gen == my) {
        if (++spins > limit || *(volatile unsigned*)&g->err) {
          atomicExch(&g->err, 1u);
          ok = false;
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok;
}

// One ready cell: pull the pushes of its higher neighbours in sweep order,
// then count down its lower neighbours.  Returns the neighbours (bit
// k = 3*(di+1) + (dj+1)) this released into the next frontier.  Values
// written by other blocks in earlier frontiers are read past L1.
__device__ unsigned drain_cell_g(const hc_view& c, const double* __restrict__ el,
                                 uint32_t cell) {
  const int W = (int)c.W;
  const int i = (int)(cell / W), j = (int)(cell % W);
  const double e = el[cell];
  // every neighbour's elevation, sweep position, area and share of its
  // area that comes here, loaded together (one round trip)
  // (elevations as their integer keys: out-of-grid entries take e's)
  const long long ke = dkey(e);
  long long ek[9];
  double an[9], gn[9];
  uint32_t pn[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int i2 = i + k / 3 - 1, j2 = j + k % 3 - 1;
    const bool in = !(i2 < 1 || i2 > c.imax || j2 < 1 || j2 > c.jmax);
    const size_t q = (size_t)i2 * W + j2;
    ek[k] = in ? dkey(__ldg(&el[q])) : ke;
    pn[k] = in ? __ldg(&c.drain_pos[q]) : 0u;
    an[k] = in ? __ldcg(&c.area[q]) : 0.0;
    gn[k] = __ldg(&c.drain_frac[(size_t)k * c.N2 + cell]);
  }
  const unsigned multi = __ldg(&c.drain_multi[cell]);
  if (pn[4] != 0) {
    double a = (e == -9999) ? 0.0 : 1.0;
    // higher neighbours the sweep reached, taken in sweep order: higher
    // elevation first, equal elevations by sorted position (only in sorted
    // runs).  Each is picked by a scan with constant indices, so the
    // neighbour values stay in registers (indexed arrays went to local
    // memory, which at this block size lives in L2).
    unsigned left = 0;
#pragma unroll
    for (int kk = 0; kk < 9; kk++)
      if (kk != 4 && ek[kk] > ke && pn[kk] != 0) left |= 1u << kk;
#pragma unroll 1
    while (left) {
      int best = -1;
      long long bk = 0;
      unsigned bp = 0;
      double aq = 0, gq = 0;
#pragma unroll
      for (int kk = 0; kk < 9; kk++) {
        if (!((left >> kk) & 1u)) continue;
        if (best < 0 || ek[kk] > bk || (ek[kk] == bk && pn[kk] > bp)) {
          best = kk;
          bk = ek[kk];
          bp = pn[kk];
          aq = an[kk];
          gq = gn[kk];
        }
      }
      left &= ~(1u << best);
      if (!((multi >> best) & 1u)) {  // one direction of q lands here
        a += aq * gq;
        continue;
      }
      const int iq = i + best / 3 - 1, jq = j + best % 3 - 1;
      const double dq = c.drain_dt[(size_t)iq * W + jq], eq = el[(size_t)iq * W + jq];
      // the directions of q whose (clamped) step lands here, in order: one
      // for an interior q, possibly more at the edges; found with integer
      // tests first, so that the divisions run once per term and not once
      // per direction of the warp's slowest lane
      unsigned dirs = 0;
#pragma unroll 1
      for (int dir = 1; dir <= 8; dir++) {
        const int i3 = clampi(iq + kDrX[dir], 1, c.imax), j3 = clampi(jq + kDrY[dir], 1, c.jmax);
        if (i3 == i && j3 == j) dirs |= 1u << dir;
      }
      while (dirs) {
        const int dir = __ffs(dirs) - 1;
        dirs &= dirs - 1;
        if (dir % 2 != 0)
          a += aq * ((eq - e) / dq);
        else
          a += aq * (((eq - e) / 1.414) / dq);
      }
    }
    if (a > 0) __stcg(&c.area[cell], a);
  }
  // No fence here: the area is read by the lower neighbours in a later
  // frontier, after a block barrier (block 0 alone) or a grid barrier, which
  // order it before those reads.
  // the eight decrements do not depend on one another: issue them together
  int old[9];
#pragma unroll
  for (int kk = 0; kk < 9; kk++) {
    const int dx = kk / 3 - 1, dy = kk % 3 - 1;
    old[kk] = (kk != 4 && ek[kk] < ke) ? atomicSub(&c.drain_pend[(i + dx) * W + (j + dy)], 1) : 0;
  }
  unsigned released = 0;
#pragma unroll
  for (int kk = 0; kk < 9; kk++) released |= (old[kk] == 1 ? 1u : 0u) << kk;
  return released;
}

// Sweeps one frontier, the threads of [start, start + stride) taking cells
// start, start + stride, ...; released cells go to fout, counted in *n_out
// (one atomic per warp).
__device__ __forceinline__ void drain_frontier(const hc_view& c, const double* __restrict__ el,
                                               const uint32_t* fin, unsigned n_in,
                                               uint32_t* fout, unsigned* n_out, unsigned start,
                                               unsigned stride) {
  const unsigned lane = threadIdx.x & 31;
  for (unsigned k0 = start - lane; k0 < n_in; k0 += stride) {
    const unsigned k = k0 + lane;
    uint32_t cell = 0;
    unsigned rel = 0;
    if (k < n_in) {
      cell = __ldcg(&fin[k]);
      rel = drain_cell_g(c, el, cell);
    }
    const unsigned cnt = __popc(rel);
    unsigned incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    unsigned base = 0;
    if (lane == 31 && incl) base = atomicAdd(n_out, incl);
    base = __shfl_sync(0xffffffffu, base, 31);
    unsigned m = base + incl - cnt;
    const int W = (int)c.W;
    while (rel) {
      const int kk = __ffs(rel) - 1;
      rel &= rel - 1;
      __stcg(&fout[m++], (uint32_t)((int)cell + (kk / 3 - 1) * W + (kk % 3 - 1)));
    }
  }
}

// All frontiers in one cooperative launch, one grid barrier between
// frontiers, or block 0 alone while they are small.  Each cell enters
// exactly one frontier, so at most imax*jmax cells are processed.
__global__ void __launch_bounds__(512, 1) k_drain_sweep(const hc_view c, hc_dev* d,
                                                      const double* __restrict__ el,
                                                      DrainSync* g) {
  __shared__ unsigned s_cnt;
  __shared__ bool s_ok;
  const unsigned nblocks = gridDim.x;
  const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned gsize = nblocks * blockDim.x;
  const unsigned long long M = (unsigned long long)c.imax * c.jmax;
  // the waits' limits (a test may shorten them and make the barrier
  // expect more arrivals than there are blocks)
  const bool test = c.wait_spins > 0;
  const long bar_limit = test ? (long)c.wait_spins : (1L << 22);
  const long solo_limit = test ? (long)c.wait_spins : (1L << 24);
  const unsigned expect = nblocks + (test ? (unsigned)c.barrier_extra : 0u);
  const unsigned solo_max = (test && c.barrier_extra > 0) ? 0u : kSoloMax;
  unsigned long long done = 0;
  unsigned level = 0;
  uint32_t* fr[2] = {c.drain_f0, c.drain_f1};
  for (;;) {
    const unsigned cur = level % 3, nxt = (level + 1) % 3;
    const unsigned n_in = *(volatile unsigned*)&g->count[cur];
    if (n_in == 0 || *(volatile unsigned*)&g->err) break;
    if (n_in <= solo_max) {
      if (blockIdx.x == 0) {
        unsigned n = n_in;
        for (;;) {
          if (threadIdx.x == 0) s_cnt = 0;
          __syncthreads();
          drain_frontier(c, el, fr[level & 1], n, fr[(level + 1) & 1], &s_cnt, threadIdx.x,
                         blockDim.x);
          __syncthreads();
          const unsigned nn = s_cnt;
          __syncthreads();  // all have read s_cnt before it is cleared
          done += n;
          level++;
          n = nn;
          if (done > M) {  // cannot happen: "higher than" has no cycles
            if (threadIdx.x == 0) atomicExch(&g->err, 2u);
            break;
          }
          if (n == 0 || n > solo_max) break;
        }
        if (threadIdx.x == 0) {
          g->count[level % 3] = n;
          g->count[(level + 1) % 3] = 0;
          g->solo_done = done;
          __threadfence();
          atomicExch(&g->solo_level, level);  // the other blocks go on from here
        }
        __syncthreads();
      } else {
        if (threadIdx.x == 0) {
          s_ok = true;
          long spins = 0;
          while (*(volatile unsigned*)&g->solo_level <= level) {
            if (++spins > solo_limit || *(volatile unsigned*)&g->err) {
              atomicExch(&g->err, 1u);
              s_ok = false;
              break;
            }
            __nanosleep(256);
          }
          __threadfence();
        }
        __syncthreads();
        if (!s_ok) break;
        level = *(volatile unsigned*)&g->solo_level;
        done = *(volatile unsigned long long*)&g->solo_done;
      }
      continue;
    }
    drain_frontier(c, el, fr[level & 1], n_in, fr[(level + 1) & 1], &g->count[nxt], gtid, gsize);
    if (gtid == 0) g->count[(level + 2) % 3] = 0;  // read two frontiers ago
    done += n_in;
    level++;
    if (done > M) {  // cannot happen: "higher than" has no cycles
      if (gtid == 0) atomicExch(&g->err, 2u);
      break;
    }
    if (!grid_barrier(g, expect, bar_limit)) break;
  }
  if (gtid == 0) {
    d->drain_done = (unsigned)done;
    d->drain_levels = level;
    d->drain_front = 0;
    if (g->err) {
      d->err_code = 401;
      d->pause |= HC_PAUSE_ERROR;
    }
  }
}

// get_catchment_input_points: cells in row-major order whose
// area*baseflow*3*DX*DX lies strictly between MIN_Q and MIN_Q_MAXVAL
__device__ __forceinline__ bool input_point(const hc_view& c, const hc_dev* d, size_t cell) {
  const int i = (int)(cell / c.W), j = (int)(cell % c.W);
  if (i < 1 || i > c.imax || j < 1 || j > c.jmax) return false;
  const double DX = c.p.DX;
  const double q = c.area[cell] * d->s.baseflow * 3 * DX * DX;
  return q > c.p.MIN_Q && q < c.p.MIN_Q_MAXVAL;
}

__global__ void __launch_bounds__(1024) k_points_count(const hc_view c, const hc_dev* d) {
  __shared__ int ws[32];
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int v = (k < c.N2 && input_point(c, d, k)) ? 1 : 0;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < 32; w++) s += ws[w];
    c.wet_sums[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(1024) k_points_scan(const hc_view c, hc_dev* d, int nblocks) {
  __shared__ int buf[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nblocks; base += 1024) {
    const int k = base + threadIdx.x;
    const int v = (k < nblocks) ? c.wet_sums[k] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const int t = (threadIdx.x >= (unsigned)off) ? buf[threadIdx.x - off] : 0;
      __syncthreads();
      buf[threadIdx.x] += t;
      __syncthreads();
    }
    if (k < nblocks) c.wet_sums[k] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) d->drain_points = (unsigned)carry;
}

__global__ void __launch_bounds__(1024) k_points_write(const hc_view c, hc_dev* d) {
  __shared__ int ws[32], wb[32];
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool v = k < c.N2 && input_point(c, d, k);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v ? 1 : 0;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < 32; w++) {
      wb[w] = s;
      s += ws[w];
    }
  }
  __syncthreads();
  if (v) {
    const int t = 1 + c.wet_sums[blockIdx.x] + wb[warp] + incl - 1;  // 1-based, as the reference
    c.cin_x[t] = (int32_t)(k / c.W);
    c.cin_y[t] = (int32_t)(k % c.W);
    const int rf = c.rfarea[k];
    if (rf >= 0 && rf <= HC_MAX_RF) atomicAdd(&d->drain_rf[rf], 1u);
  }
}

// totalinputpoints and catchment_input_counter (entries 1..rfnum restart
// from zero; an rfarea of 0 keeps adding to entry 0, as in the reference)
__global__ void k_points_finish(const hc_view c, hc_dev* d) {
  hc_scalars& s = d->s;
  for (int n = 1; n <= c.p.rfnum && n <= HC_MAX_RF; n++) s.catchment_input_counter[n] = 0;
  for (int n = 0; n <= HC_MAX_RF; n++) {
    if (n <= c.p.rfnum) s.catchment_input_counter[n] += (double)d->drain_rf[n];
    d->drain_rf[n] = 0;
  }
  const unsigned t = d->drain_points;
  s.totalinputpoints = (t == 0) ? 1.0 : (double)t;
}

}  // namespace

// The drainage area for the elevations `el` (device), then the input points.
// `sort_order` is called, and its order used, only when the sort's order
// among equal elevations can show (see the top of the file).  Returns HC_OK,
// or HC_ERR_CUDA; *sorted tells which way it went.
hc_status run_drainage_device(hc_ctx* c, const double* el, bool area_valid,
                              hc_status (*sort_order)(hc_ctx*, const double*, uint32_t*),
                              bool* sorted) {
  hc_view& v = c->v;
  const size_t N2 = v.N2;
  cudaStream_t s = c->s;
  *sorted = false;
  if (!area_valid) {
    const unsigned long long M = (unsigned long long)v.imax * v.jmax;
    const unsigned long long P = N2 - M;
    hc_drain_aux a0;
    std::memset(&a0, 0, sizeof a0);
    a0.min_u = ~0ull;
    a0.k = P;
    if (cudaMemcpyAsync(v.drain_aux, &a0, sizeof a0, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return HC_ERR_CUDA;
    dim3 b(32, 8);
    dim3 g((v.jmax + 31) / 32, (v.imax + 7) / 8);
    k_drain_min<<<g, b, 0, s>>>(v, el);
    k_drain_mincount<<<g, b, 0, s>>>(v, el);
    for (int shift = 56; shift >= 0; shift -= 8) {
      k_sel_hist<<<g, b, 0, s>>>(v, el, shift);
      k_sel_pick<<<1, 1, 0, s>>>(v, shift, P);
    }
    k_drain_init<<<g, b, 0, s>>>(v, c->dev, el);
    k_drain_frac<<<g, b, 0, s>>>(v, el);
    c->launches += 20;
    hc_drain_aux a;
    if (cudaMemcpyAsync(&a, v.drain_aux, sizeof a, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return HC_ERR_CUDA;
    c->d2h_bytes += sizeof a;
    const bool top_ok = a.gt == P - 1 || (a.prefix == kZeroKey && a.real_eq == 0);
    const bool bottom_ok =
        a.min_u > kZeroKey || (a.min_u < kZeroKey && (a.min_count == 1 || !a.min_matters));
    if (a.contrib_tie || !top_ok || !bottom_ok) {
      if (sort_order(c, el, v.drain_f1) != HC_OK) return HC_ERR_CUDA;
      if (cudaMemsetAsync(v.drain_pos, 0, N2 * 4, s) != cudaSuccess) return HC_ERR_CUDA;
      k_drain_pos<<<152 * 4, 256, 0, s>>>(v, v.drain_f1);
      c->launches += 1;
      *sorted = true;
    }
    // the sweep: all blocks resident (cooperative launch), grid barriers
    // between frontiers
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // one block per SM: fewer arrivals at each barrier; a frontier averages a
    // few thousand cells
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_drain_sweep, 512, 0);
    const int nblocks = std::max(1, sms * std::min(per_sm, 1));
    // the barrier lives in the selection's histogram, which is finished
    static_assert(sizeof(DrainSync) <= sizeof(hc_drain_aux::hist), "barrier fits");
    DrainSync* gs = (DrainSync*)((char*)v.drain_aux + offsetof(hc_drain_aux, hist));
    const unsigned* front = (const unsigned*)((const char*)c->dev + offsetof(hc_dev, drain_front));
    if (cudaMemsetAsync(gs, 0, sizeof(DrainSync), s) != cudaSuccess ||
        cudaMemcpyAsync((char*)gs + offsetof(DrainSync, count), front, sizeof(unsigned),
                        cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return HC_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    const double* elp = el;
    hc_dev* devp = c->dev;
    void* args[] = {(void*)&v, (void*)&devp, (void*)&elp, (void*)&gs};
    const cudaError_t le = cudaLaunchCooperativeKernel((const void*)k_drain_sweep, nblocks, 512,
                                                       args, 0, s);
    cudaEventRecord(e1, s);
    c->launches += 1;
    if (le != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return HC_ERR_CUDA;
    }
    if (cudaEventSynchronize(e1) == cudaSuccess) {
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      c->stat_n[HC_STAT_DRAINAGE_SWEEP]++;
      c->stat_ms[HC_STAT_DRAINAGE_SWEEP] += ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  const int nb = (int)((N2 + 1023) / 1024);
  k_points_count<<<nb, 1024, 0, s>>>(v, c->dev);
  k_points_scan<<<1, 1024, 0, s>>>(v, c->dev, nb);
  k_points_write<<<nb, 1024, 0, s>>>(v, c->dev);
  k_points_finish<<<1, 1, 0, s>>>(v, c->dev);
  c->launches += 4;
  return cudaGetLastError() == cudaSuccess ? HC_OK : HC_ERR_CUDA;
}
