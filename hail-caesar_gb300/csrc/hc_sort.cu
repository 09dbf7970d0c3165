// The order in which drainage_area_D8 (LSDCatchmentModel.cpp:2091-2271)
// sweeps the cells: the permutation std::sort gives the reference's
// (key, elevation) pairs, compared by elevation only (:2143-2180), ties
// included, computed on the device.
//
// std::sort in GCC's library is introsort (Musser, "Introspective Sorting
// and Selection Algorithms", 1997): while a range holds more than 16
// elements, move the median of (first+1, middle, last-1) to `first`, split
// [first+1, last) around it with the two-sided unguarded partition, recurse
// into the right part and loop on the left, each with one level less of a
// depth budget of 2*floor(log2 n); a range that exhausts the budget is
// heap-sorted; a final insertion sort runs over the whole array.  Every step
// below is that algorithm's step, element for element; only the order in
// which independent ranges are processed differs, which cannot change the
// result.
//
// The partition is the one sequential piece.  Its left pointer stops at
// elements >= pivot ("left stoppers" L1 < L2 < ...), its right pointer at
// elements <= pivot ("right stoppers" R1 > R2 > ..., from the right), and
// pair k is swapped while Lk < Rk.  Since Lk < Rk exactly when at least k
// right stoppers lie right of Lk, the number of swaps K, the pairs, and the
// returned cut min(L(K+1), RK) follow from two prefix counts, so a range is
// split in parallel with the result of the serial loop.  After the loop
// every run between two cuts holds at most 16 elements, everything left of
// a cut is <= everything right of it, and the final insertion sort (strict
// comparisons) therefore amounts to a stable sort of each run.
//
// Ranges longer than kLocalMax are split level by level by the whole grid
// (chunks of kChunk elements, one block each); shorter ones are finished by
// one block each in shared memory, a warp per range.  A range that runs out
// of depth budget (adversarial inputs, never seen on terrain) or a NaN
// elevation make the caller fall back to the host's exact sort.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

#include "../../include/hc_gpu.h"
#include "hc_internal.cuh"

namespace {

constexpr int kRun = 16;          // std::sort's insertion-sort threshold
constexpr int kLocalMax = 4096;   // ranges finished by one block
constexpr int kChunk = 2048;      // elements per block in the grid-wide splits
constexpr int kChunkThreads = 256;
constexpr int kChunkRounds = kChunk / kChunkThreads;
constexpr int kLocalThreads = 256;
constexpr int kLocalLists = 256;  // ranges > 16 within kLocalMax elements: at most 240

struct SortRange {
  uint32_t first, last;
  int32_t depth, pad;
};

struct SortCtl {
  unsigned n_next;    // ranges appended for the next grid-wide level
  unsigned n_local;   // ranges for the block phase
  unsigned fallback;  // depth budget exhausted, NaN key, or a list full
  unsigned pad;
};

}  // namespace

struct hc_sort_work {
  size_t cap = 0;  // elements
  size_t max_g = 0, max_l = 0, max_chunks = 0;
  long long* key = nullptr;
  uint32_t* idx = nullptr;
  uint32_t* posL = nullptr;
  uint32_t* posR = nullptr;
  SortRange* glist[2] = {nullptr, nullptr};
  SortRange* llist = nullptr;
  uint32_t* chunk_base = nullptr;  // per range of the level, + total
  uint32_t* cnt = nullptr;         // per chunk: left stoppers, right stoppers
  uint32_t* off = nullptr;         // their exclusive scans (+ sentinel)
  uint32_t* kcnt = nullptr;        // per range: swaps
  SortCtl* ctl = nullptr;
  SortCtl* ctl_h = nullptr;        // pinned
};

namespace {

__device__ __forceinline__ void swap_at(long long* k, uint32_t* ix, size_t a, size_t b) {
  const long long t = k[a];
  k[a] = k[b];
  k[b] = t;
  const uint32_t u = ix[a];
  ix[a] = ix[b];
  ix[b] = u;
}

// __move_median_to_first(result, a, b, c)
template <typename I>
__device__ __forceinline__ void median_to_first(long long* k, uint32_t* ix, I result, I a, I b,
                                                I c) {
  if (k[a] < k[b]) {
    if (k[b] < k[c]) swap_at(k, ix, result, b);
    else if (k[a] < k[c]) swap_at(k, ix, result, c);
    else swap_at(k, ix, result, a);
  } else if (k[a] < k[c]) {
    swap_at(k, ix, result, a);
  } else if (k[b] < k[c]) {
    swap_at(k, ix, result, c);
  } else {
    swap_at(k, ix, result, b);
  }
}

// ------------------------------------------------------------ the inputs
// drainage_area_D8's pair vector: (imax+2)(jmax+2) pairs, (0, 0) except
// positions 1 .. imax*jmax, which hold the cells row by row (:2104-2146)
__global__ void k_sort_fill_drainage(const hc_view c, const double* __restrict__ el,
                                     long long* key, uint32_t* idx, SortCtl* ctl) {
  const size_t M = (size_t)c.imax * c.jmax;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < c.N2;
       k += (size_t)gridDim.x * blockDim.x) {
    long long kk = 0;
    uint32_t cell = 0;
    if (k >= 1 && k <= M) {
      const size_t i = (k - 1) / c.jmax + 1, j = (k - 1) % c.jmax + 1;
      cell = (uint32_t)(i * c.W + j);
      const double e = el[cell];
      if (disnan(e)) atomicOr(&ctl->fallback, 1u);
      kk = dkey(e);
    }
    key[k] = kk;
    idx[k] = cell;
  }
}

__global__ void k_sort_fill_values(const double* __restrict__ v, size_t n, long long* key,
                                   uint32_t* idx, SortCtl* ctl) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    if (disnan(v[k])) atomicOr(&ctl->fallback, 1u);
    key[k] = dkey(v[k]);
    idx[k] = (uint32_t)k;
  }
}

// ------------------------------------------------- block-wide helpers
// exclusive scan of one value per thread (blockDim.x == 1024 or 256);
// returns the exclusive prefix, *total the block's sum
template <int NT>
__device__ __forceinline__ unsigned block_exscan(unsigned x, unsigned* total) {
  __shared__ unsigned warp_sum[NT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned v = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) warp_sum[w] = v;
  __syncthreads();
  if (w == 0) {
    unsigned s = (lane < NT / 32) ? warp_sum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < NT / 32) warp_sum[lane] = s;
  }
  __syncthreads();
  const unsigned before = (w > 0 ? warp_sum[w - 1] : 0) + v - x;
  *total = warp_sum[NT / 32 - 1];
  __syncthreads();
  return before;
}

// ------------------------------------------------ grid-wide split, per level
// Median-of-three for every range of the level and its number of chunks;
// chunk_base = exclusive scan of those (one block).
__global__ void __launch_bounds__(1024) k_sort_pivots(hc_sort_work w, int cur, unsigned nR) {
  const SortRange* R = w.glist[cur];
  if (threadIdx.x == 0) w.ctl->n_next = 0;
  unsigned carry = 0;
  for (unsigned base = 0; base < nR; base += 1024) {
    const unsigned r = base + threadIdx.x;
    unsigned ch = 0;
    if (r < nR) {
      const SortRange g = R[r];
      w.kcnt[r] = 0;
      if (g.depth == 0) {
        atomicOr(&w.ctl->fallback, 1u);  // std::sort would heap-sort this range
      } else {
        const size_t f = g.first, l = g.last;
        median_to_first<size_t>(w.key, w.idx, f, f + 1, f + (l - f) / 2, l - 1);
        ch = (unsigned)((l - f - 1 + kChunk - 1) / kChunk);
      }
    }
    unsigned tot;
    const unsigned ex = block_exscan<1024>(ch, &tot);
    if (r < nR) w.chunk_base[r] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) w.chunk_base[nR] = carry;
}

// the range a chunk belongs to: the last r with chunk_base[r] <= c
__device__ __forceinline__ unsigned range_of(const uint32_t* cb, unsigned nR, unsigned c) {
  unsigned lo = 0, hi = nR;  // cb[lo] <= c < cb[hi]
  while (hi - lo > 1) {
    const unsigned mid = (lo + hi) >> 1;
    if (cb[mid] <= c) lo = mid;
    else hi = mid;
  }
  return lo;
}

// stoppers per chunk
__global__ void __launch_bounds__(kChunkThreads) k_sort_count(hc_sort_work w, int cur,
                                                              unsigned nR) {
  const unsigned c = blockIdx.x;
  if (c >= w.chunk_base[nR]) return;
  const unsigned r = range_of(w.chunk_base, nR, c);
  const SortRange g = w.glist[cur][r];
  const long long p = w.key[g.first];
  const size_t base = (size_t)g.first + 1 + (size_t)(c - w.chunk_base[r]) * kChunk;
  const size_t end = base + kChunk < (size_t)g.last ? base + kChunk : (size_t)g.last;
  unsigned nl = 0, nr = 0;
#pragma unroll
  for (int q = 0; q < kChunkRounds; q++) {
    const size_t x = base + (size_t)q * kChunkThreads + threadIdx.x;
    if (x < end) {
      const long long k = w.key[x];
      nl += (k >= p);
      nr += (k <= p);
    }
  }
  unsigned tl, tr;
  block_exscan<kChunkThreads>(nl, &tl);
  block_exscan<kChunkThreads>(nr, &tr);
  if (threadIdx.x == 0) {
    w.cnt[2 * c] = tl;
    w.cnt[2 * c + 1] = tr;
  }
}

// exclusive scans of the chunk counts (one block), sentinel at the end
__global__ void __launch_bounds__(1024) k_sort_scan(hc_sort_work w, unsigned nR) {
  const unsigned T = w.chunk_base[nR];
  unsigned cl = 0, cr = 0;
  for (unsigned base = 0; base < T; base += 1024) {
    const unsigned c = base + threadIdx.x;
    const unsigned a = (c < T) ? w.cnt[2 * c] : 0, b = (c < T) ? w.cnt[2 * c + 1] : 0;
    unsigned ta, tb;
    const unsigned ea = block_exscan<1024>(a, &ta);
    const unsigned eb = block_exscan<1024>(b, &tb);
    if (c < T) {
      w.off[2 * c] = cl + ea;
      w.off[2 * c + 1] = cr + eb;
    }
    cl += ta;
    cr += tb;
  }
  if (threadIdx.x == 0) {
    w.off[2 * T] = cl;
    w.off[2 * T + 1] = cr;
  }
}

// ranks of the stoppers: posL[first + k - 1] = Lk, posR[first + k - 1] = Rk;
// kcnt[r] += the left stoppers with at least their rank of right stoppers
// to their right (those are L1 .. LK)
__global__ void __launch_bounds__(kChunkThreads) k_sort_rank(hc_sort_work w, int cur,
                                                             unsigned nR) {
  const unsigned c = blockIdx.x;
  if (c >= w.chunk_base[nR]) return;
  const unsigned r = range_of(w.chunk_base, nR, c);
  const SortRange g = w.glist[cur][r];
  const long long p = w.key[g.first];
  const unsigned c0 = w.chunk_base[r], c1 = w.chunk_base[r + 1];
  const size_t base = (size_t)g.first + 1 + (size_t)(c - c0) * kChunk;
  const size_t end = base + kChunk < (size_t)g.last ? base + kChunk : (size_t)g.last;
  unsigned carryL = w.off[2 * c] - w.off[2 * c0];
  unsigned carryR = w.off[2 * c + 1] - w.off[2 * c0 + 1];
  const unsigned totR = w.off[2 * c1 + 1] - w.off[2 * c0 + 1];
  unsigned swaps = 0;
  for (int q = 0; q < kChunkRounds; q++) {
    const size_t x = base + (size_t)q * kChunkThreads + threadIdx.x;
    bool isL = false, isR = false;
    if (x < end) {
      const long long k = w.key[x];
      isL = k >= p;
      isR = k <= p;
    }
    unsigned tl, tr;
    const unsigned el = block_exscan<kChunkThreads>(isL, &tl);
    const unsigned er = block_exscan<kChunkThreads>(isR, &tr);
    const unsigned kL = carryL + el + 1;     // rank if a left stopper
    const unsigned rleq = carryR + er + isR;  // right stoppers at or before x
    if (isL) {
      w.posL[g.first + kL - 1] = (uint32_t)x;
      swaps += (totR - rleq >= kL);
    }
    if (isR) w.posR[g.first + (totR - rleq)] = (uint32_t)x;
    carryL += tl;
    carryR += tr;
  }
  unsigned ts;
  block_exscan<kChunkThreads>(swaps, &ts);
  if (threadIdx.x == 0 && ts) atomicAdd(&w.kcnt[r], ts);
}

// the K swaps of every range
__global__ void __launch_bounds__(kChunkThreads) k_sort_swap(hc_sort_work w, int cur,
                                                             unsigned nR) {
  const unsigned c = blockIdx.x;
  if (c >= w.chunk_base[nR]) return;
  const unsigned r = range_of(w.chunk_base, nR, c);
  const SortRange g = w.glist[cur][r];
  const unsigned K = w.kcnt[r];
  const unsigned k0 = (c - w.chunk_base[r]) * kChunk;
  for (unsigned k = k0 + threadIdx.x; k < K && k < k0 + kChunk; k += kChunkThreads)
    swap_at(w.key, w.idx, w.posL[g.first + k], w.posR[g.first + k]);
}

// the cut of every range; children longer than kLocalMax go to the next
// level, the others to the block phase
__global__ void __launch_bounds__(1024) k_sort_split(hc_sort_work w, int cur, unsigned nR) {
  for (unsigned r = threadIdx.x; r < nR; r += 1024) {
    const SortRange g = w.glist[cur][r];
    if (g.depth == 0) continue;
    const unsigned c0 = w.chunk_base[r], c1 = w.chunk_base[r + 1];
    const unsigned totL = w.off[2 * c1] - w.off[2 * c0];
    const unsigned K = w.kcnt[r];
    uint32_t cut = (K < totL) ? w.posL[g.first + K] : 0xffffffffu;
    if (K > 0) cut = min(cut, w.posR[g.first + K - 1]);
    if (!(cut > g.first && cut < g.last)) {  // cannot happen; never trust it
      atomicOr(&w.ctl->fallback, 1u);
      continue;
    }
    const SortRange kids[2] = {{g.first, cut, g.depth - 1, 0}, {cut, g.last, g.depth - 1, 0}};
    for (const SortRange& k : kids) {
      if (k.last - k.first > (uint32_t)kLocalMax) {
        const unsigned s = atomicAdd(&w.ctl->n_next, 1u);
        if (s < w.max_g) w.glist[cur ^ 1][s] = k;
        else atomicOr(&w.ctl->fallback, 1u);
      } else {
        const unsigned s = atomicAdd(&w.ctl->n_local, 1u);
        if (s < w.max_l) w.llist[s] = k;
        else atomicOr(&w.ctl->fallback, 1u);
      }
    }
  }
}

// ------------------------------------------------------- block phase
struct LocalRange {
  uint16_t first, last;
  int16_t depth, pad;
};

// One warp splits [f, l) of the block's shared copy; returns the cut.
__device__ unsigned warp_split(long long* sk, uint32_t* si, uint16_t* pL, uint16_t* pR,
                               unsigned f, unsigned l) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1;
  if (lane == 0) median_to_first<unsigned>(sk, si, f, f + 1, f + (l - f) / 2, l - 1);
  __syncwarp();
  const long long p = sk[f];
  unsigned nr = 0;
  for (unsigned x = f + 1 + lane; x < l; x += 32) nr += (sk[x] <= p);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nr += __shfl_xor_sync(0xffffffffu, nr, o);
  const unsigned totR = nr;
  unsigned baseL = 0, baseR = 0, K = 0;
  for (unsigned x0 = f + 1; x0 < l; x0 += 32) {
    const unsigned x = x0 + lane;
    const bool valid = x < l;
    const long long k = valid ? sk[x] : 0;
    const bool isL = valid && k >= p, isR = valid && k <= p;
    const unsigned bL = __ballot_sync(0xffffffffu, isL), bR = __ballot_sync(0xffffffffu, isR);
    const unsigned kL = baseL + __popc(bL & lt) + 1;
    const unsigned rleq = baseR + __popc(bR & lt) + isR;
    bool sw = false;
    if (isL) {
      pL[f + kL - 1] = (uint16_t)x;
      sw = totR - rleq >= kL;
    }
    if (isR) pR[f + (totR - rleq)] = (uint16_t)x;
    K += __popc(__ballot_sync(0xffffffffu, sw));
    baseL += __popc(bL);
    baseR += __popc(bR);
  }
  __syncwarp();
  unsigned cut = (K < baseL) ? pL[f + K] : 0xffffffffu;
  if (K > 0) cut = min(cut, (unsigned)pR[f + K - 1]);
  for (unsigned k = lane; k < K; k += 32) swap_at(sk, si, pL[f + k], pR[f + k]);
  __syncwarp();
  return cut;
}

__global__ void __launch_bounds__(kLocalThreads) k_sort_local(hc_sort_work w, uint32_t* out) {
  extern __shared__ __align__(16) unsigned char smem[];
  long long* sk = (long long*)smem;
  uint32_t* si = (uint32_t*)(sk + kLocalMax);
  uint16_t* pL = (uint16_t*)(si + kLocalMax);
  uint16_t* pR = pL + kLocalMax;
  unsigned* marks = (unsigned*)(pR + kLocalMax);
  LocalRange* lists = (LocalRange*)(marks + kLocalMax / 32);
  __shared__ unsigned nlist[2], bad;
  const SortRange g = w.llist[blockIdx.x];
  const unsigned m = g.last - g.first;
  for (unsigned x = threadIdx.x; x < m; x += kLocalThreads) {
    sk[x] = w.key[g.first + x];
    si[x] = w.idx[g.first + x];
  }
  for (unsigned x = threadIdx.x; x < kLocalMax / 32; x += kLocalThreads) marks[x] = 0;
  if (threadIdx.x == 0) {
    bad = 0;
    nlist[0] = 0;
    if (m > kRun) {
      lists[0] = {0, (uint16_t)m, (int16_t)g.depth, 0};
      nlist[0] = 1;
    }
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int a = 0;; a ^= 1) {
    const unsigned na = nlist[a];
    if (na == 0) break;
    if (threadIdx.x == 0) nlist[a ^ 1] = 0;
    __syncthreads();
    LocalRange* A = lists + a * kLocalLists;
    LocalRange* B = lists + (a ^ 1) * kLocalLists;
    for (unsigned rr = warp; rr < na; rr += kLocalThreads / 32) {
      const LocalRange q = A[rr];
      if (q.depth == 0) {  // std::sort would heap-sort this range
        if (lane == 0) bad = 1;
        continue;
      }
      const unsigned cut = warp_split(sk, si, pL, pR, q.first, q.last);
      if (lane == 0) {
        if (!(cut > q.first && cut < q.last)) {
          bad = 1;
          continue;
        }
        atomicOr(&marks[cut >> 5], 1u << (cut & 31));
        if (cut - q.first > kRun) {
          const unsigned s = atomicAdd(&nlist[a ^ 1], 1u);
          if (s < kLocalLists) B[s] = {q.first, (uint16_t)cut, (int16_t)(q.depth - 1), 0};
          else bad = 1;
        }
        if (q.last - cut > kRun) {
          const unsigned s = atomicAdd(&nlist[a ^ 1], 1u);
          if (s < kLocalLists) B[s] = {(uint16_t)cut, q.last, (int16_t)(q.depth - 1), 0};
          else bad = 1;
        }
      }
    }
    __syncthreads();
    if (bad) break;
  }
  __syncthreads();
  if (bad) {
    if (threadIdx.x == 0) atomicOr(&w.ctl->fallback, 1u);
    return;
  }
  // the final insertion sort, run by run (stable within each run)
  for (unsigned s = threadIdx.x; s < m; s += kLocalThreads) {
    if (s != 0 && !((marks[s >> 5] >> (s & 31)) & 1u)) continue;
    unsigned e = s + 1;
    while (e < m && !((marks[e >> 5] >> (e & 31)) & 1u)) e++;
    for (unsigned i = s + 1; i < e; i++) {
      const long long v = sk[i];
      const uint32_t vi = si[i];
      unsigned j = i;
      while (j > s && v < sk[j - 1]) {
        sk[j] = sk[j - 1];
        si[j] = si[j - 1];
        j--;
      }
      sk[j] = v;
      si[j] = vi;
    }
  }
  __syncthreads();
  for (unsigned x = threadIdx.x; x < m; x += kLocalThreads) out[g.first + x] = si[x];
}

constexpr size_t kLocalSmem = (size_t)kLocalMax * (8 + 4 + 2 + 2) + kLocalMax / 8 +
                              2 * kLocalLists * sizeof(LocalRange);

template <typename T>
cudaError_t grow(T** p, size_t n) {
  if (*p) cudaFree(*p);
  *p = nullptr;
  return cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
}

}  // namespace

hc_sort_work* sort_work_new() { return new hc_sort_work(); }

void sort_work_free(hc_sort_work* w) {
  if (!w) return;
  cudaFree(w->key);
  cudaFree(w->idx);
  cudaFree(w->posL);
  cudaFree(w->posR);
  cudaFree(w->glist[0]);
  cudaFree(w->glist[1]);
  cudaFree(w->llist);
  cudaFree(w->chunk_base);
  cudaFree(w->cnt);
  cudaFree(w->off);
  cudaFree(w->kcnt);
  cudaFree(w->ctl);
  cudaFreeHost(w->ctl_h);
  delete w;
}

static cudaError_t reserve(hc_sort_work* w, size_t n) {
  if (n <= w->cap && w->ctl) return cudaSuccess;
  const int depth0 = n > 1 ? 2 * (63 - __builtin_clzll((unsigned long long)n)) : 0;
  w->max_g = n / (kLocalMax + 1) + 1;
  // every level splits at most max_g ranges, two children each
  w->max_l = 2 * w->max_g * (size_t)(depth0 + 1) + 1;
  w->max_chunks = n / kChunk + w->max_g + 1;
  cudaError_t e;
  if ((e = grow(&w->key, n)) != cudaSuccess || (e = grow(&w->idx, n)) != cudaSuccess ||
      (e = grow(&w->posL, n)) != cudaSuccess || (e = grow(&w->posR, n)) != cudaSuccess ||
      (e = grow(&w->glist[0], w->max_g)) != cudaSuccess ||
      (e = grow(&w->glist[1], w->max_g)) != cudaSuccess ||
      (e = grow(&w->llist, w->max_l)) != cudaSuccess ||
      (e = grow(&w->chunk_base, w->max_g + 1)) != cudaSuccess ||
      (e = grow(&w->cnt, 2 * w->max_chunks)) != cudaSuccess ||
      (e = grow(&w->off, 2 * w->max_chunks + 2)) != cudaSuccess ||
      (e = grow(&w->kcnt, w->max_g)) != cudaSuccess || (e = grow(&w->ctl, 1)) != cudaSuccess)
    return e;
  if (!w->ctl_h && (e = cudaMallocHost((void**)&w->ctl_h, sizeof(SortCtl))) != cudaSuccess)
    return e;
  w->cap = n;
  return cudaSuccess;
}

// Sorts the n keys in w->key (with w->idx) as std::sort would; the
// permutation goes to `out` (device, n entries).  *fallback: the host must
// sort instead (out is then undefined).  Synchronises `s`.
static cudaError_t sort_run(hc_sort_work* w, size_t n, uint32_t* out, cudaStream_t s,
                            bool* fallback, int64_t* launches) {
  *fallback = false;
  if (n == 0) return cudaSuccess;
  if (n > 0xffffffffull) {
    *fallback = true;
    return cudaSuccess;
  }
  const int depth0 = n > 1 ? 2 * (63 - __builtin_clzll((unsigned long long)n)) : 0;
  const SortRange all = {0, (uint32_t)n, depth0, 0};
  cudaError_t e;
  unsigned nR = 0;
  SortCtl h = {0, 0, 0, 0};
  if (n > (size_t)kLocalMax) {
    if ((e = cudaMemcpyAsync(w->glist[0], &all, sizeof all, cudaMemcpyHostToDevice, s)) !=
        cudaSuccess)
      return e;
    nR = 1;
  } else {
    if ((e = cudaMemcpyAsync(w->llist, &all, sizeof all, cudaMemcpyHostToDevice, s)) !=
        cudaSuccess)
      return e;
    h.n_local = 1;
  }
  // the fill kernel may have flagged a NaN already: keep that flag
  if ((e = cudaMemcpyAsync(&w->ctl->n_next, &h.n_next, 2 * sizeof(unsigned),
                           cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return e;
  const hc_sort_work wv = *w;
  int cur = 0;
  while (nR > 0) {
    const unsigned tmax = (unsigned)(n / kChunk + nR + 1);
    k_sort_pivots<<<1, 1024, 0, s>>>(wv, cur, nR);
    k_sort_count<<<tmax, kChunkThreads, 0, s>>>(wv, cur, nR);
    k_sort_scan<<<1, 1024, 0, s>>>(wv, nR);
    k_sort_rank<<<tmax, kChunkThreads, 0, s>>>(wv, cur, nR);
    k_sort_swap<<<tmax, kChunkThreads, 0, s>>>(wv, cur, nR);
    k_sort_split<<<1, 1024, 0, s>>>(wv, cur, nR);
    *launches += 6;
    if ((e = cudaMemcpyAsync(w->ctl_h, w->ctl, sizeof(SortCtl), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return e;
    if (w->ctl_h->fallback) {
      *fallback = true;
      return cudaSuccess;
    }
    nR = w->ctl_h->n_next;
    cur ^= 1;
  }
  const unsigned nl = (nR == 0 && n > (size_t)kLocalMax) ? w->ctl_h->n_local : h.n_local;
  static bool attr = false;
  if (!attr) {
    if ((e = cudaFuncSetAttribute(k_sort_local, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kLocalSmem)) != cudaSuccess)
      return e;
    attr = true;
  }
  if (nl > 0) {
    k_sort_local<<<nl, kLocalThreads, kLocalSmem, s>>>(wv, out);
    *launches += 1;
  }
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpyAsync(w->ctl_h, w->ctl, sizeof(SortCtl), cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return e;
  *fallback = w->ctl_h->fallback != 0;
  return cudaSuccess;
}

cudaError_t device_drainage_order(hc_ctx* c, const double* el, uint32_t* order, bool* fallback) {
  if (!c->sort_work) c->sort_work = sort_work_new();
  hc_sort_work* w = c->sort_work;
  const size_t n = c->v.N2;
  cudaError_t e = reserve(w, n);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(w->ctl, 0, sizeof(SortCtl), c->s)) != cudaSuccess) return e;
  k_sort_fill_drainage<<<152 * 4, 256, 0, c->s>>>(c->v, el, w->key, w->idx, w->ctl);
  c->launches += 1;
  return sort_run(w, n, order, c->s, fallback, &c->launches);
}

cudaError_t device_sort_values(hc_sort_work* w, const double* v, size_t n, uint32_t* perm,
                               cudaStream_t s, bool* fallback, int64_t* launches) {
  cudaError_t e = reserve(w, n);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(w->ctl, 0, sizeof(SortCtl), s)) != cudaSuccess) return e;
  if (n > 0) {
    k_sort_fill_values<<<152 * 4, 256, 0, s>>>(v, n, w->key, w->idx, w->ctl);
    *launches += 1;
  }
  return sort_run(w, n, perm, s, fallback, launches);
}

extern "C" hc_status hc_drainage_sort(const double* values, uint64_t n, uint32_t* perm,
                                      int32_t* on_device) {
  if (on_device) *on_device = 1;
  if (n == 0) return HC_OK;
  if (!values || !perm || n > 0xffffffffull) return HC_ERR_ARG;
  hc_sort_work* w = sort_work_new();
  double* dv = nullptr;
  uint32_t* dp = nullptr;
  cudaStream_t s = nullptr;
  bool fallback = false;
  int64_t launches = 0;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void**)&dv, n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&dp, n * sizeof(uint32_t));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dv, values, n * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = device_sort_values(w, dv, n, dp, s, &fallback, &launches);
  if (e == cudaSuccess && !fallback)
    e = cudaMemcpyAsync(perm, dp, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(dv);
  cudaFree(dp);
  sort_work_free(w);
  if (s) cudaStreamDestroy(s);
  if (e != cudaSuccess) return HC_ERR_CUDA;
  if (fallback) {
    std::vector<std::pair<double, double>> pr(n);
    for (uint64_t k = 0; k < n; k++) pr[k] = std::make_pair((double)k, values[k]);
    host_sort_exact(pr.data(), n, 16);
    for (uint64_t k = 0; k < n; k++) perm[k] = (uint32_t)pr[k].first;
    if (on_device) *on_device = 0;
  }
  return HC_OK;
}
