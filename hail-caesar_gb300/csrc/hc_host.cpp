// Host-side pieces of the path that the reference itself runs rarely and
// that depend only on inputs or on a full sort:
//   * drainage area + catchment input points (drainage_area_D8 :2091-2271,
//     zero_and_calc_drainage_area :2072-2089, get_catchment_input_points
//     :3741-3767), recomputed when the baseflow threshold moves;
//   * the TOPMODEL recurrence (topmodel_runoff :3649-3715), which depends
//     only on the rain table and is tabulated once per run.
// Both use the host C library exactly as the reference does (std::sort with
// the same comparator on the same vectors; glibc exp/log), so their results
// are the reference's bit for bit.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

#include "../../include/hc_gpu.h"

namespace {
const int kDX[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1};
const int kDY[9] = {0, -1, -1, 0, 1, 1, 1, 0, -1};
}

// The reference sorts the row keys and the column keys of all cells in two
// separate std::sort calls on (key, elevation) pairs.  std::sort's moves
// depend only on the comparisons, which see only the elevations, so both
// calls apply the same permutation: one sort carrying the cell number gives
// both orders, ties included.  The permutation is kept and reused while the
// elevations are unchanged (always in hydro-only runs).
struct DrainageCache {
  std::vector<uint32_t> order;   // cell numbers in the reference's processing order
  std::vector<double> elev;      // elevations the order was made from
};

void* host_drainage_cache_new() { return new DrainageCache(); }
void host_drainage_cache_free(void* p) { delete (DrainageCache*)p; }

void host_drainage_and_points(const hc_params* p, const double* elev, const int32_t* rfarea,
                              double baseflow, double* area, int32_t* cin_x, int32_t* cin_y,
                              int* total, double* counters, void* cache_p, bool elev_fixed) {
  const unsigned imax = p->imax, jmax = p->jmax;
  const size_t W = jmax + 2, N2 = (size_t)(imax + 2) * W;
  auto ix = [&](unsigned i, unsigned j) { return (size_t)i * W + j; };
  DrainageCache* cache = (DrainageCache*)cache_p;
  bool reuse = cache && !cache->order.empty();
  if (reuse && !elev_fixed)
    reuse = std::memcmp(cache->elev.data(), elev, N2 * sizeof(double)) == 0;
  if (!reuse) {
    std::vector<std::pair<double, double>> pr(N2);
    for (size_t k = 0; k < N2; k++) pr[k] = std::make_pair(0.0, 0.0);
    size_t inc = 1;
    for (unsigned i = 1; i <= imax; i++)
      for (unsigned j = 1; j <= jmax; j++) {
        pr[inc] = std::make_pair((double)ix(i, j), elev[ix(i, j)]);
        inc++;
      }
    std::sort(pr.begin(), pr.end(),
              [](const std::pair<double, double>& a, const std::pair<double, double>& b) {
                return a.second < b.second;
              });
    cache->order.resize(N2);
    for (size_t k = 0; k < N2; k++) cache->order[k] = (uint32_t)pr[k].first;
    cache->elev.assign(elev, elev + N2);
  }
  std::vector<double> ad(N2, 0.0);
  for (unsigned i = 1; i <= imax; i++)
    for (unsigned j = 1; j <= jmax; j++) {
      ad[ix(i, j)] = 1;
      area[ix(i, j)] = 0;
      if (elev[ix(i, j)] == -9999) ad[ix(i, j)] = 0.0;
    }
  const std::vector<uint32_t>& ord = cache->order;
  for (unsigned n = jmax * imax; n >= 1; n--) {
    const int i = (int)(ord[n] / W), j = (int)(ord[n] % W);
    double& a = ad[ix(i, j)];
    if (!(a > 0)) continue;
    if (a > area[ix(i, j)]) area[ix(i, j)] = a;
    const double e = elev[ix(i, j)];
    double difftot = 0;
    int nb[9][2];
    for (int dir = 1; dir <= 8; dir++) {
      int j2 = j + kDY[dir], i2 = i + kDX[dir];
      if (j2 < 1) j2 = 1;
      if (i2 < 1) i2 = 1;
      if (j2 > (int)jmax) j2 = jmax;
      if (i2 > (int)imax) i2 = imax;
      nb[dir][0] = i2;
      nb[dir][1] = j2;
      const double e2 = elev[ix(i2, j2)];
      if (dir % 2 != 0) {
        if (e2 < e) difftot += e - e2;
      } else {
        if (e2 < e) difftot += (e - e2) / 1.414;
      }
    }
    if (difftot > 0) {
      for (int dir = 1; dir <= 8; dir++) {
        const int i2 = nb[dir][0], j2 = nb[dir][1];
        const double e2 = elev[ix(i2, j2)];
        if (dir % 2 != 0) {
          if (e2 < e) ad[ix(i2, j2)] += a * ((e - e2) / difftot);
        } else {
          if (e2 < e) ad[ix(i2, j2)] += a * (((e - e2) / 1.414) / difftot);
        }
      }
    }
    a = 0;
  }
  // input points: cin_x/cin_y keep their old contents beyond the new count,
  // as the reference's vectors do
  const double DX = p->DX;
  int t = 0;
  for (int n = 1; n <= p->rfnum; n++) counters[n] = 0;
  for (unsigned i = 1; i <= imax; i++)
    for (unsigned j = 1; j <= jmax; j++) {
      const double q = area[ix(i, j)] * baseflow * 3 * DX * DX;
      if (q > p->MIN_Q && q < p->MIN_Q_MAXVAL) {
        t++;
        cin_x[t] = i;
        cin_y[t] = j;
        counters[rfarea[ix(i, j)]] += 1;
      }
    }
  if (t == 0) t = 1;
  *total = t;
}

void host_topmodel_table(const hc_params* p, const float* rain, int rows, int cols, int nsteps,
                         double* table) {
  const int rf = p->rfnum;
  std::vector<double> jv(rf + 1, 0.000000001), jo(rf + 1, 0.000000001);
  std::vector<double> oldm(rf + 1, 0.0), newm(rf + 1, 0.0);
  const double M = p->M;
  auto step = [&](double cyc) {
    const int ts = (int)(cyc / p->rain_data_time_step);
    for (int n = 1; n <= rf; n++) {
      double lrr = 0;
      const double fts = 60;
      oldm[n] = newm[n];
      jo[n] = jv[n];
      float v = 0.0f;
      if (ts >= 0 && ts < rows && n - 1 < cols) v = rain[(size_t)ts * cols + (n - 1)];
      if (v > 0) lrr = p->rain_factor * ((v / 1000) / 3600);
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

// global_landsliding :5529-5654.  A serial relaxation over the whole grid
// (x outer, y inner; every test sees the moves before it; up to 200 sweeps
// until nothing moves).  It changes elevations only and runs once a
// simulated day, so it runs here on the host, in the reference's order,
// on a downloaded copy of elev.  Returns the number of sweeps.
int host_global_landsliding(const hc_params* p, const double* bedrock, double* elev) {
  const unsigned imax = p->imax, jmax = p->jmax;
  const size_t W = jmax + 2;
  const double factor = std::tan((p->failureangle * (3.141592654 / 180))) * p->DX;
  const double active = p->active, EF = p->ERODEFACTOR;
  static const int ox[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  static const int oy[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  unsigned inc = 0;
  double total = 0;
  do {
    total = 0;
    inc++;
    for (unsigned x = 2; x < imax; x++)
      for (unsigned y = 2; y < jmax; y++) {
        const size_t c = (size_t)x * W + y;
        double wet_factor = factor;
        if (elev[c] <= (bedrock[c] + active)) wet_factor = 10 * p->DX;
        for (int k = 0; k < 8; k++) {
          const size_t nb = (size_t)(x + ox[k]) * W + (y + oy[k]);
          const bool diag = (ox[k] != 0 && oy[k] != 0);
          const double drop = diag ? ((elev[c] - elev[nb]) / 1.41) : (elev[c] - elev[nb]);
          if (drop > wet_factor && elev[nb] > -9999) {
            double diff = (diag ? ((elev[c] - elev[nb]) / 1.41) : (elev[c] - elev[nb])) - wet_factor;
            if ((elev[c] - diff) < (bedrock[c] + active)) diff = (elev[c] - (bedrock[c] + active));
            if (diff > EF) diff = EF;
            elev[c] -= diff;
            elev[nb] += diff;
            total += diff;
          }
        }
      }
  } while (total > 0 && inc < 200);
  return (int)inc;
}
