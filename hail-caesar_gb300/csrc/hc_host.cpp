// Host-side pieces of the path that the reference itself runs rarely and
// that depend only on inputs or on a full sort:
//   * the processing order of the drainage area (drainage_area_D8
//     :2091-2271), a sort of all elevations, recomputed when the baseflow
//     threshold moves (the accumulation itself runs on the device,
//     hc_drain.cu);
//   * the TOPMODEL recurrence (topmodel_runoff :3649-3715), which depends
//     only on the rain table and is tabulated once per run.
// Both use the host C library exactly as the reference does (std::sort with
// the same comparator on the same vectors; glibc exp/log), so their results
// are the reference's bit for bit.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/hc_gpu.h"

// The reference sorts the row keys and the column keys of all cells in two
// separate std::sort calls on (key, elevation) pairs, comparing elevations
// only (drainage_area_D8 :2091-2180).  std::sort's moves depend only on the
// comparisons, which see only the elevations, so both calls apply the same
// permutation: one sort carrying the cell number gives both orders, ties
// included.
//
// That permutation, including the order it gives to equal elevations, is
// what GCC's std::sort produces: introsort (Musser, "Introspective Sorting
// and Selection Algorithms", 1997) with median-of-three pivots, a two-sided
// partition, heapsort below a depth of 2*floor(log2 n), and a final
// insertion sort over runs of at most 16.  sort_exact below performs exactly
// those steps; only the independent sub-ranges left of and right of each cut
// are sorted by separate threads, which cannot change the result.  A CPU test
// checks the permutation against std::sort on inputs with many ties.
namespace exact_sort {

using Pair = std::pair<double, double>;  // (cell number, elevation)
constexpr std::ptrdiff_t kRun = 16;

inline bool before(const Pair& a, const Pair& b) { return a.second < b.second; }

// median of *a, *b, *c moved to *result
inline void median_to_first(Pair* result, Pair* a, Pair* b, Pair* c) {
  if (before(*a, *b)) {
    if (before(*b, *c)) std::swap(*result, *b);
    else if (before(*a, *c)) std::swap(*result, *c);
    else std::swap(*result, *a);
  } else if (before(*a, *c)) {
    std::swap(*result, *a);
  } else if (before(*b, *c)) {
    std::swap(*result, *c);
  } else {
    std::swap(*result, *b);
  }
}

// partition of [first, last) around *pivot (which lies before first)
inline Pair* split_at(Pair* first, Pair* last, const Pair* pivot) {
  for (;;) {
    while (before(*first, *pivot)) ++first;
    --last;
    while (before(*pivot, *last)) --last;
    if (!(first < last)) return first;
    std::swap(*first, *last);
    ++first;
  }
}

inline void insertion_run(Pair* first, Pair* last) {
  for (Pair* i = first + 1; i < last; ++i) {
    Pair v = *i;
    Pair* j = i;
    while (j > first && before(v, *(j - 1))) {
      *j = *(j - 1);
      --j;
    }
    *j = v;
  }
}

inline void heap_run(Pair* first, Pair* last) {
  auto cmp = [](const Pair& a, const Pair& b) { return a.second < b.second; };
  std::make_heap(first, last, cmp);
  std::sort_heap(first, last, cmp);
}

// The introsort loop on [first, last).  Right-hand ranges of at least
// `spawn_min` elements go to a new thread while `spawn` threads remain.
void loop(Pair* first, Pair* last, long depth, int spawn, std::ptrdiff_t spawn_min,
          std::vector<std::thread>* threads, std::mutex* mu) {
  while (last - first > kRun) {
    if (depth == 0) {
      heap_run(first, last);
      return;
    }
    --depth;
    Pair* mid = first + (last - first) / 2;
    median_to_first(first, first + 1, mid, last - 1);
    Pair* cut = split_at(first + 1, last, first);
    if (spawn > 0 && last - cut >= spawn_min) {
      const int child = spawn / 2;
      spawn -= child + 1;
      std::lock_guard<std::mutex> lock(*mu);
      threads->emplace_back(loop, cut, last, depth, child, spawn_min, threads, mu);
    } else {
      loop(cut, last, depth, 0, spawn_min, threads, mu);
    }
    last = cut;
  }
  // the final insertion sort, restricted to this run: no element moves past
  // a cut (everything left of a cut is <= the pivot <= everything right)
  insertion_run(first, last);
}

}  // namespace exact_sort

void host_sort_exact(std::pair<double, double>* a, size_t n, int threads) {
  if (n < 2) return;
  long lg = 0;
  for (size_t m = n; m > 1; m >>= 1) lg++;
  std::vector<std::thread> th;
  th.reserve(2 * threads + 2);
  std::mutex mu;
  exact_sort::loop(a, a + n, 2 * lg, threads - 1, 1 << 16, &th, &mu);
  // joined in creation order; a thread may add more while we wait
  for (size_t k = 0;; k++) {
    std::thread t;
    {
      std::lock_guard<std::mutex> lock(mu);
      if (k >= th.size()) break;
      t = std::move(th[k]);
    }
    t.join();
  }
}

// The processing order of drainage_area_D8 for these elevations: order[n]
// is the cell at sorted position n (0 for the reference's padding pairs).
// Kept and reused while the elevations are unchanged (always in hydro-only
// runs).
struct DrainageCache {
  std::vector<uint32_t> order;
  std::vector<double> elev;      // elevations the order was made from
};

void* host_drainage_cache_new() { return new DrainageCache(); }
void host_drainage_cache_free(void* p) { delete (DrainageCache*)p; }

const uint32_t* host_drainage_order(const hc_params* p, const double* elev, void* cache_p,
                                    bool* reused) {
  const unsigned imax = p->imax, jmax = p->jmax;
  const size_t W = jmax + 2, N2 = (size_t)(imax + 2) * W;
  DrainageCache* cache = (DrainageCache*)cache_p;
  *reused = !cache->order.empty() &&
            std::memcmp(cache->elev.data(), elev, N2 * sizeof(double)) == 0;
  if (*reused) return cache->order.data();
  // the reference's pair vector: (imax+2)(jmax+2) pairs, (0, 0) except
  // positions 1 .. imax*jmax, which hold the cells row by row
  std::vector<std::pair<double, double>> pr(N2, std::make_pair(0.0, 0.0));
  size_t inc = 1;
  for (unsigned i = 1; i <= imax; i++)
    for (unsigned j = 1; j <= jmax; j++) {
      const size_t cell = (size_t)i * W + j;
      pr[inc++] = std::make_pair((double)cell, elev[cell]);
    }
  unsigned hw = std::thread::hardware_concurrency();
  host_sort_exact(pr.data(), N2, (int)std::max(1u, std::min(hw, 16u)));
  cache->order.resize(N2);
  for (size_t k = 0; k < N2; k++) cache->order[k] = (uint32_t)pr[k].first;
  cache->elev.assign(elev, elev + N2);
  return cache->order.data();
}

void host_topmodel_table(const hc_params* p, const float* rain, int rows, int cols, int nsteps,
                         double* table) {
  const int rf = p->rfnum;
  std::vector<double> jv(rf + 1, 0.000000001), jo(rf + 1, 0.000000001);
  std::vector<double> oldm(rf + 1, 0.0), newm(rf + 1, 0.0);
  const double M = p->M;
  const bool grid = p->spatially_complex_rainfall != 0;
  auto rain_at = [&](int ts, int col) {
    return (ts >= 0 && ts < rows && col >= 0 && col < cols) ? rain[(size_t)ts * cols + col] : 0.0f;
  };
  auto step = [&](double cyc) {
    const int ts = (int)(cyc / p->rain_data_time_step);
    for (int n = grid ? 0 : 1; n <= rf; n++) {
      double lrr = 0;
      const double fts = 60;
      oldm[n] = newm[n];
      jo[n] = jv[n];
      if (grid) {
        // runoffGrid::calculate_runoff (LSDRainfallRunoff.cpp:175-241) for
        // rain state n: the grid holds the rain as a double, rain_factor is
        // passed as an int; state 0 gets no rain (rainGrid::create :33-66)
        double g = 0;
        if (rf == 1) g = (n == 1) ? (double)rain_at(ts, 0) : 0.0;
        else if (n >= 1 && n <= rf - 1) g = (double)rain_at(ts, n - 1);
        if (g > 0) lrr = (int)p->rain_factor * ((g / 1000) / 3600);
      } else {
        const float v = rain_at(ts, n - 1);
        if (v > 0) lrr = p->rain_factor * ((v / 1000) / 3600);
      }
      const double j0 = jo[n];
      if (lrr == 0) {
        jv[n] = j0 / (1 + ((j0 * fts) / M));
        newm[n] = M / fts * std::log(1 + ((j0 * fts) / M));
      }
      if (lrr > 0) {
        jv[n] = lrr / (((lrr - j0) / j0) * std::exp((0 - lrr) * fts / M) + 1);
        newm[n] = (M / fts) * std::log(((lrr - j0) + j0 * std::exp((lrr * fts) / M)) / lrr);
      }
      if (newm[n] < 0) newm[n] = 0;
    }
  };
  for (int t = 0; t < nsteps; t++) {
    step(t == 0 ? 1.0 : (double)t);  // call 0 is initialise_rainfall_runoff's topmodel_runoff(1.0)
    double* row = table + (size_t)t * 2 * (rf + 1);
    for (int n = 0; n <= rf; n++) {
      row[n] = oldm[n];
      row[(rf + 1) + n] = newm[n];
    }
  }
}

// Derivatives of the TOPMODEL table (host_topmodel_table) with respect to the
// rain table, by forward-mode differentiation of the same recurrence: for
// table rows t < nsteps, zone n (1..rfnum) and rain row k < rows,
//   d_old[(t*(rf+1) + n)*rows + k] = d old_j_mean[n] / d rain[k][n-1]
//   d_new[...]                     = d new_j_mean[n] / d rain[k][n-1].
// A rain value of 0 sits on the switch between the recession and the
// infiltration formulas; its derivative is taken as 0.
void host_topmodel_tangent(const hc_params* p, const float* rain, int rows, int cols, int nsteps,
                           double* d_old, double* d_new) {
  const int rf = p->rfnum;
  const double M = p->M, fts = 60, a = fts / M;
  const size_t R = (size_t)rows;
  std::fill(d_old, d_old + (size_t)nsteps * (rf + 1) * R, 0.0);
  std::fill(d_new, d_new + (size_t)nsteps * (rf + 1) * R, 0.0);
  for (int n = 1; n <= rf; n++) {
    double jv = 0.000000001, newm = 0.0;
    std::vector<double> dj(R, 0.0), dnew(R, 0.0), dold(R, 0.0), djo(R, 0.0);
    for (int t = 0; t < nsteps; t++) {
      const double cyc = (t == 0) ? 1.0 : (double)t;
      const int ts = (int)(cyc / p->rain_data_time_step);
      dold = dnew;
      djo = dj;
      const double j0 = jv;
      float v = 0.0f;
      if (ts >= 0 && ts < rows && n - 1 < cols) v = rain[(size_t)ts * cols + (n - 1)];
      double lrr = 0;
      if (v > 0) lrr = p->rain_factor * ((v / 1000) / 3600);
      const double dlrr = (v > 0) ? p->rain_factor / 3600000.0 : 0.0;  // d lrr / d v
      if (lrr == 0) {
        const double q = 1 + j0 * a;
        jv = j0 / (1 + ((j0 * fts) / M));
        newm = M / fts * std::log(1 + ((j0 * fts) / M));
        for (size_t k = 0; k < R; k++) {
          dj[k] = djo[k] / (q * q);
          dnew[k] = djo[k] / q;
        }
      } else {
        const double E = std::exp((0 - lrr) * fts / M);
        const double u = ((lrr - j0) / j0) * E + 1;
        const double eP = std::exp((lrr * fts) / M);
        const double X = (lrr - j0) + j0 * eP;
        jv = lrr / u;
        newm = (M / fts) * std::log(X / lrr);
        for (size_t k = 0; k < R; k++) {
          const double dl = (k == (size_t)ts) ? dlrr : 0.0;
          const double d0 = djo[k];
          const double du = E * (dl / j0 - lrr / (j0 * j0) * d0) + (lrr / j0 - 1) * E * (-a * dl);
          dj[k] = dl / u - lrr / (u * u) * du;
          const double dX = dl - d0 + d0 * eP + j0 * eP * a * dl;
          dnew[k] = (1 / a) * (dX / X - dl / lrr);
        }
      }
      if (newm < 0) {
        newm = 0;
        std::fill(dnew.begin(), dnew.end(), 0.0);
      }
      double* ro = d_old + ((size_t)t * (rf + 1) + n) * R;
      double* rn = d_new + ((size_t)t * (rf + 1) + n) * R;
      for (size_t k = 0; k < R; k++) {
        ro[k] = dold[k];
        rn[k] = dnew[k];
      }
    }
  }
}
