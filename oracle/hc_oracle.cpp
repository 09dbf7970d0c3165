// CPU restatement of HAIL-CAESAR's per-timestep raster path.
//
// TEST INFRASTRUCTURE: the parity checker for the GPU product and the CPU
// baseline timed by bench.py.  Never linked into the product.
//
// Every function states the reference member it restates
// (src/catchmentmodel/LSDCatchmentModel.cpp:line unless said otherwise).
// Arithmetic keeps the reference's evaluation order and its float/double and
// int/double promotions, because the goal is bit-identical FP64 results
// against the reference's own serial build (oracle/ref_harness.cpp).  The
// code structure (flat arrays, index helpers, one struct) is this project's.
//
// Built twice by oracle/Makefile: serial (parity) and with -DHCO_OPENMP, which
// enables OpenMP on the same loops the reference parallelises (timing only).

#include "hc_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#ifdef HCO_OPENMP
#include <omp.h>
#define HCO_PRAGMA(x) _Pragma(#x)
#else
#define HCO_PRAGMA(x)
#endif

namespace {

constexpr double kGravity = 9.81;                          // .hpp:438
constexpr int kDX[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1};     // .hpp:445 deltaX
constexpr int kDY[9] = {0, -1, -1, 0, 1, 1, 1, 0, -1};     // .hpp:446 deltaY
constexpr unsigned G = HC_G_MAX;                           // G_MAX = 10
constexpr double kNoData = -9999;

// static_cast<int>(double) as x86-64 executes it (cvttsd2si): NaN and values
// outside the int range give INT_MIN.  call_erosion :2283 converts
// ERODEFACTOR/tempbmax, which is +inf whenever nothing was entrained; the
// reference's own build runs on x86-64, where that yields INT_MIN and so
// erode_mult = 1.  (aarch64 saturates to INT_MAX instead, giving 5.)
inline int x86_trunc_to_int(double v) {
  if (!(v > -2147483649.0 && v < 2147483648.0)) return (int)0x80000000u;
  return (int)v;
}

}  // namespace

struct hco_model {
  hc_params p;
  unsigned imax, jmax;
  double DX;
  size_t W;  // padded row length jmax+2
  size_t N2; // (imax+2)(jmax+2)

  std::vector<double> elev, water_depth, qx, qy, qxs, qys, Vsusptot, Vel, Tau,
      bedrock, spat_var_mannings, area, area_depth, ss, tempcreep;
  std::vector<double> vel_dir;         // N2 * 9
  std::vector<double> sr, sl, su, sd;  // N2 * 10
  std::vector<double> grain;           // nrec * 11
  std::vector<double> strata;          // nrec * 10 * 11
  std::vector<int32_t> index, down_scan, rfarea;
  std::vector<uint8_t> listed;  // membership of down_scan (the ledger's mask-edge term)
  std::vector<uint8_t> inputpointsarray;
  std::vector<double> edge, edge2, veg;  // (imax+1)(jmax+1) [*4]
  std::vector<int32_t> cin_x, cin_y;
  std::vector<std::vector<float>> rain;
  std::vector<std::vector<float>> reach[HC_MAX_POINTS];

  double mannings;
  double cycle = 0, previous = 0, time_step = 1, maxdepth = 10;
  double waterinput = 0, waterOut = 0, iod = 0, temptot = 0;
  // water ledger of the current iteration (sums of depth, m): added by the
  // inputs to rows 1..imax / columns 1..jmax, taken off the edges by
  // water_flux_out, zeroed at no-data cells by depth_update; and the depth
  // sum of the grid at the last scan_area with its iteration
  double vin_it = 0, vout_it = 0, vlost_it = 0, vmask_it = 0, vol_scan = 0;
  long vol_scan_counter = -1;
  bool on_grid(long i, long j) const { return i >= 1 && i <= imax && j >= 1 && j <= jmax; }
  int counter = 0;
  double erode_call = 0, erode_mult = 1, lateralcounter = 1;
  double time_1 = 1, baseflow = 0, sediQ = 0, globalsediq = 0, tempbmax = 0;
  double creep_time = 1, creep_time2 = 1;
  int grain_array_tot = 1;
  // a record beyond the grain arrays' N2/LIMIT rows was asked for (the
  // reference's arrays would overflow); hco_iterate stops
  bool grain_full = false;
  int totalinputpoints = 0;
  std::vector<double> sum_grain, jv, jo, j_mean, old_j_mean, new_j_mean;
  // runoffGrid (LSDRainfallRunoff.cpp:120-133), per cell, for the
  // distributed TOPMODEL (spatially_complex_rainfall)
  std::vector<double> rj, rjo, rjm, rold, rnew;
  std::vector<int> nActualGridCells, cin_counter;

  inline size_t ix(unsigned i, unsigned j) const { return (size_t)i * W + j; }
  inline size_t ex(unsigned i, unsigned j) const { return (size_t)i * (jmax + 1) + j; }
  inline double& E(unsigned i, unsigned j) { return elev[ix(i, j)]; }
  inline double& H(unsigned i, unsigned j) { return water_depth[ix(i, j)]; }
  inline int32_t& IDX(unsigned i, unsigned j) { return index[ix(i, j)]; }
  inline double& GR(int rec, unsigned n) { return grain[(size_t)rec * 11 + n]; }
  inline double& ST(int rec, unsigned z, unsigned n) {
    return strata[((size_t)rec * 10 + z) * 11 + n];
  }
  inline int32_t& DS(unsigned col, unsigned k) {
    return down_scan[(size_t)col * (imax + 2) + k];
  }
  inline double& VD(unsigned i, unsigned j, unsigned n) { return vel_dir[ix(i, j) * 9 + n]; }
  inline double& S4(std::vector<double>& a, unsigned i, unsigned j, unsigned n) {
    return a[ix(i, j) * 10 + n];
  }
  inline double& EDGE(unsigned i, unsigned j) { return edge[ex(i, j)]; }
  inline double& VEG(unsigned i, unsigned j, unsigned k) { return veg[ex(i, j) * 4 + k]; }
  inline double Dsize(unsigned n) const { return p.d[n]; }
};

// ---------------------------------------------------------------------------
// construction: initialise_arrays :1617 + zero_values :2891
// ---------------------------------------------------------------------------
extern "C" hco_model* hco_create(const hc_params* prm) {
  hco_model* m = new hco_model();
  m->p = *prm;
  m->imax = prm->imax;
  m->jmax = prm->jmax;
  m->DX = prm->DX;
  m->W = m->jmax + 2;
  m->N2 = (size_t)(m->imax + 2) * m->W;
  const size_t N2 = m->N2;
  m->elev.assign(N2, kNoData);
  m->water_depth.assign(N2, 0.0);
  m->qx.assign(N2, 0.0);
  m->qy.assign(N2, 0.0);
  m->qxs.assign(N2, 0.0);
  m->qys.assign(N2, 0.0);
  m->Vsusptot.assign(N2, 0.0);
  m->Vel.assign(N2, 0.0);
  m->Tau.assign(N2, 0.0);
  m->bedrock.assign(N2, kNoData);
  m->spat_var_mannings.assign(N2, 0.0);
  m->area.assign(N2, 0.0);
  m->area_depth.assign(N2, 0.0);
  m->ss.assign(N2, 0.0);
  m->tempcreep.assign(N2, 0.0);
  m->vel_dir.assign(N2 * 9, 0.0);
  if (!prm->hydro_only) {  // only erosion runs allocate these (:1752-1762)
    m->sr.assign(N2 * 10, 0.0);
    m->sl.assign(N2 * 10, 0.0);
    m->su.assign(N2 * 10, 0.0);
    m->sd.assign(N2 * 10, 0.0);
    size_t nrec = N2 / (size_t)std::max(1, prm->LIMIT);
    m->grain.assign(nrec * 11, 0.0);
    m->strata.assign(nrec * 10 * 11, 0.0);
  }
  m->index.assign(N2, -9999);
  m->down_scan.assign((size_t)(m->jmax + 2) * (m->imax + 2), 0);
  m->rfarea.assign(N2, 1);
  m->inputpointsarray.assign(N2, 0);
  m->edge.assign((size_t)(m->imax + 1) * (m->jmax + 1), 0.0);
  m->edge2.assign((size_t)(m->imax + 1) * (m->jmax + 1), 0.0);
  m->veg.assign((size_t)(m->imax + 1) * (m->jmax + 1) * 4, 0.0);
  m->cin_x.assign((size_t)m->imax * m->jmax + 2, 0);
  m->cin_y.assign((size_t)m->imax * m->jmax + 2, 0);
  m->mannings = prm->mannings;
  m->baseflow = prm->baseflow;
  const int rf = prm->rfnum;
  m->sum_grain.assign(G + 1, 0.0);
  m->jv.assign(rf + 1, 0.000000001);
  m->jo.assign(rf + 1, 0.000000001);
  m->j_mean.assign(rf + 1, 0.0);
  m->old_j_mean.assign(rf + 1, 0.0);
  m->new_j_mean.assign(rf + 1, 0.0);
  m->nActualGridCells.assign(rf + 1, 0);
  if (prm->spatially_complex_rainfall) {
    m->rj.assign(m->N2, 0.000000001);
    m->rjo.assign(m->N2, 0.000000001);
    m->rjm.assign(m->N2, 0.0);
    m->rold.assign(m->N2, 0.0);
    m->rnew.assign(m->N2, 0.0);
  }
  m->cin_counter.assign(rf + 1, 0);
  // The reach block of initialise_arrays marks the input cells in
  // inputpointsarray (:1770), but zero_values (:2905), called at the end of
  // initialise_arrays, clears the whole array again; the mask is therefore
  // all false in every run and suspended sediment settles on input cells too.
  return m;
}

extern "C" void hco_destroy(hco_model* m) { delete m; }

extern "C" void hco_set_rain(hco_model* m, const float* rain, int rows, int cols) {
  m->rain.assign(rows, std::vector<float>(cols));
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < cols; c++) m->rain[r][c] = rain[(size_t)r * cols + c];
}

extern "C" void hco_set_reach(hco_model* m, int point, const float* d, int rows, int cols) {
  m->reach[point].assign(rows, std::vector<float>(cols));
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < cols; c++) m->reach[point][r][c] = d[(size_t)r * cols + c];
}

// ---------------------------------------------------------------------------
// timestep control :1873-1933
// ---------------------------------------------------------------------------
static double cfl(hco_model* m) {  // courant_friedrichs_lewy_condition :1884
  return m->p.courant_number * (m->DX / std::sqrt(kGravity * (m->maxdepth)));
}

extern "C" void hco_set_maximum_timestep(hco_model* m) {  // :1890-1910
  if (m->maxdepth <= 0.1) m->maxdepth = 0.1;
  if (m->time_step < cfl(m)) m->time_step = cfl(m);
  if (m->iod > m->p.in_out_difference_allowed && m->time_step > cfl(m))
    m->time_step = cfl(m);
}

extern "C" double hco_get_flow_timestep(hco_model* m) {  // :1913-1923
  double f = m->time_step;
  if (f > cfl(m)) f = cfl(m);
  return f;
}

// ---------------------------------------------------------------------------
// drainage area and catchment input points :2055-2271, :3741-3767
// ---------------------------------------------------------------------------
// The permutation the reference's sort of (key, elevation) pairs applies
// (:2143-2180, std::sort with LSDUtils::sort_pair_second): perm[k] = the
// index of the value at sorted position k.  The same library call.
extern "C" void hco_sort_perm(const double* v, int64_t n, uint32_t* perm) {
  std::vector<std::pair<double, double>> pr((size_t)n);
  for (int64_t k = 0; k < n; k++) pr[(size_t)k] = std::make_pair((double)k, v[k]);
  std::sort(pr.begin(), pr.end(), [](const std::pair<double, double>& a,
                                     const std::pair<double, double>& b) {
    return a.second < b.second;
  });
  for (int64_t k = 0; k < n; k++) perm[k] = (uint32_t)pr[(size_t)k].first;
}

static void drainage_area_D8(hco_model* m) {  // :2091-2271
  const unsigned imax = m->imax, jmax = m->jmax;
  const size_t N2 = m->N2;
  std::vector<double> tv(N2, 0.0), tv2(N2, 0.0), xkey(N2, 0.0), ykey(N2, 0.0);
  int inc = 1;
  for (unsigned i = 1; i <= imax; i++)
    for (unsigned j = 1; j <= jmax; j++) {
      tv[inc] = m->E(i, j);
      xkey[inc] = i;
      inc++;
    }
  // The reference sorts (key, elevation) pairs by elevation with std::sort
  // and LSDUtils::sort_pair_second; ties are ordered by std::sort itself, so
  // the same library call on the same vectors is used here.
  auto by_second = [](const std::pair<double, double>& a,
                      const std::pair<double, double>& b) { return a.second < b.second; };
  std::vector<std::pair<double, double>> xp(N2), yp(N2);
  for (size_t k = 0; k < N2; k++) xp[k] = std::make_pair(xkey[k], tv[k]);
  std::sort(xp.begin(), xp.end(), by_second);
  inc = 1;
  for (unsigned i = 1; i <= imax; i++)
    for (unsigned j = 1; j <= jmax; j++) {
      tv2[inc] = m->E(i, j);
      ykey[inc] = j;
      inc++;
    }
  for (size_t k = 0; k < N2; k++) yp[k] = std::make_pair(ykey[k], tv2[k]);
  std::sort(yp.begin(), yp.end(), by_second);

  for (unsigned n = jmax * imax; n >= 1; n--) {
    int i = (int)xp[n].first;
    int j = (int)yp[n].first;
    double& ad = m->area_depth[m->ix(i, j)];
    if (ad > 0) {
      if (ad > m->area[m->ix(i, j)]) m->area[m->ix(i, j)] = ad;
      double difftot = 0;
      const double e = m->E(i, j);
      for (int dir = 1; dir <= 8; dir++) {
        int j2 = j + kDY[dir], i2 = i + kDX[dir];
        if (j2 < 1) j2 = 1;
        if (i2 < 1) i2 = 1;
        if (j2 > (int)jmax) j2 = jmax;
        if (i2 > (int)imax) i2 = imax;
        double e2 = m->E(i2, j2);
        if (dir % 2 != 0) {
          if (e2 < e) difftot += e - e2;
        } else {
          if (e2 < e) difftot += (e - e2) / 1.414;
        }
      }
      if (difftot > 0) {
        for (int dir = 1; dir <= 8; dir++) {
          int i2 = i + kDX[dir], j2 = j + kDY[dir];
          if (j2 < 1) j2 = 1;
          if (i2 < 1) i2 = 1;
          if (j2 > (int)jmax) j2 = jmax;
          if (i2 > (int)imax) i2 = imax;
          double e2 = m->E(i2, j2);
          if (dir % 2 != 0) {
            if (e2 < e) m->area_depth[m->ix(i2, j2)] += ad * ((e - e2) / difftot);
          } else {
            if (e2 < e)
              m->area_depth[m->ix(i2, j2)] += ad * (((e - e2) / 1.414) / difftot);
          }
        }
      }
      ad = 0;
    }
  }
}

static void zero_and_calc_drainage_area(hco_model* m) {  // :2072-2089
  for (unsigned i = 1; i <= m->imax; i++)
    for (unsigned j = 1; j <= m->jmax; j++) {
      m->area_depth[m->ix(i, j)] = 1;
      m->area[m->ix(i, j)] = 0;
      if (m->E(i, j) == -9999) m->area_depth[m->ix(i, j)] = 0.0;
    }
  drainage_area_D8(m);
}

static void get_catchment_input_points(hco_model* m) {  // :3741-3767
  const double DX = m->DX;
  m->totalinputpoints = 0;
  for (int n = 1; n <= m->p.rfnum; n++) m->cin_counter[n] = 0;
  for (unsigned i = 1; i <= m->imax; i++)
    for (unsigned j = 1; j <= m->jmax; j++) {
      double q = m->area[m->ix(i, j)] * m->baseflow * 3 * DX * DX;
      if (q > m->p.MIN_Q && q < m->p.MIN_Q_MAXVAL) {
        m->totalinputpoints++;
        m->cin_x[m->totalinputpoints] = i;
        m->cin_y[m->totalinputpoints] = j;
        m->cin_counter[m->rfarea[m->ix(i, j)]]++;
      }
    }
  if (m->totalinputpoints == 0) m->totalinputpoints = 1;
}

// ---------------------------------------------------------------------------
// TOPMODEL rainfall-runoff, uniform / zoned rain :3649-3724
// ---------------------------------------------------------------------------
static float rain_at(hco_model* m, int row, int col) {
  if (row < 0 || row >= (int)m->rain.size()) return 0.0f;
  if (col < 0 || col >= (int)m->rain[row].size()) return 0.0f;
  return m->rain[row][col];
}

static void topmodel_runoff(hco_model* m, double cyc) {  // :3649-3715
  int ts = (int)(cyc / m->p.rain_data_time_step);
  const double M = m->p.M;
  for (int n = 1; n <= m->p.rfnum; n++) {
    double lrr = 0;
    const double fts = 60;
    m->old_j_mean[n] = m->new_j_mean[n];
    m->jo[n] = m->jv[n];
    float v = rain_at(m, ts, n - 1);
    if (v > 0) lrr = m->p.rain_factor * ((v / 1000) / 3600);  // float arithmetic
    const double jo = m->jo[n];
    if (lrr == 0) {
      m->jv[n] = jo / (1 + ((jo * fts) / M));
      m->new_j_mean[n] = M / fts * std::log(1 + ((jo * fts) / M));
    }
    if (lrr > 0) {
      m->jv[n] = lrr / (((lrr - jo) / jo) * std::exp((0 - lrr) * fts / M) + 1);
      m->new_j_mean[n] =
          (M / fts) * std::log(((lrr - jo) + jo * std::exp((lrr * fts) / M)) / lrr);
    }
    if (m->new_j_mean[n] < 0) m->new_j_mean[n] = 0;
  }
}

static void calchydrograph(hco_model* m, double t) {  // :3718-3724
  for (int n = 1; n <= m->p.rfnum; n++)
    m->j_mean[n] = m->old_j_mean[n] + (((m->new_j_mean[n] - m->old_j_mean[n]) / 2) * (2 - t));
}

// Distributed TOPMODEL (spatially_complex_rainfall).  rainGrid::create
// (LSDRainfallRunoff.cpp:33-66): one zone: every cell (padding included)
// takes column 0; otherwise the cells of zones 1 .. rfnum-1 take their
// column and the others none (the loop stops before rfnum).
static void rain_grid(hco_model* m, int ts, std::vector<double>& g) {
  g.assign(m->N2, 0.0);
  const int rf = m->p.rfnum;
  if (rf == 1) {
    std::fill(g.begin(), g.end(), (double)rain_at(m, ts, 0));
    return;
  }
  for (unsigned i = 1; i < m->imax; i++)
    for (unsigned j = 1; j < m->jmax; j++)
      for (int z = 1; z < rf; z++)
        if (m->rfarea[m->ix(i, j)] == z) g[m->ix(i, j)] = rain_at(m, ts, z - 1);
}

// topmodel_runoff(cycle, runoff) :3610-3628 -> runoffGrid::calculate_runoff
// (LSDRainfallRunoff.cpp:175-241), which takes rain_factor as an int
static void topmodel_runoff_grid(hco_model* m, double cyc) {
  const int ts = (int)(cyc / m->p.rain_data_time_step);
  std::vector<double> g;
  rain_grid(m, ts, g);
  const int rain_factor = (int)m->p.rain_factor;
  const double M = m->p.M;
  for (unsigned a = 1; a < m->imax; a++)
    for (unsigned b = 1; b < m->jmax; b++) {
      const size_t c = m->ix(a, b);
      if (!(m->E(a, b) > -9999)) continue;
      double lrr = 0;
      const double lts = 60;
      m->rold[c] = m->rnew[c];
      m->rjo[c] = m->rj[c];
      if (g[c] > 0) lrr = rain_factor * ((g[c] / 1000) / 3600);
      const double jo = m->rjo[c];
      if (lrr == 0) {
        m->rj[c] = jo / (1 + ((jo * lts) / M));
        m->rnew[c] = M / lts * std::log(1 + ((jo * lts) / M));
      }
      if (lrr > 0) {
        m->rj[c] = lrr / (((lrr - jo) / jo) * std::exp((0 - lrr) * lts / M) + 1);
        m->rnew[c] = (M / lts) * std::log(((lrr - jo) + jo * std::exp((lrr * lts) / M)) / lrr);
      }
      if (m->rnew[c] < 0) m->rnew[c] = 0;
    }
}

static void calchydrograph_grid(hco_model* m, double t) {  // :3728-3740
  for (unsigned a = 1; a <= m->imax; a++)
    for (unsigned b = 1; b <= m->jmax; b++) {
      const size_t c = m->ix(a, b);
      m->rjm[c] = m->rold[c] + (((m->rnew[c] - m->rold[c]) / 2) * (2 - t));
    }
}

// catchment_water_input_and_hydrology(flow_timestep, runoff) :3544-3607
static void catchment_water_input_grid(hco_model* m, double fdt) {
  const double DX = m->DX;
  for (unsigned i = 1; i < m->imax; i++)
    for (unsigned j = 1; j < m->jmax; j++) m->waterinput += m->rjm[m->ix(i, j)] * DX * DX;
  for (unsigned i = 1; i < m->imax; i++)
    for (unsigned j = 1; j < m->jmax; j++) {
      double amt = m->rjm[m->ix(i, j)] * fdt;
      if (amt > m->p.ERODEFACTOR) amt = m->p.ERODEFACTOR;
      m->waterinput += (amt / fdt) * DX * DX;
      m->H(i, j) += amt;
      m->vin_it += amt;
    }
  double new_jmeanmax = 0;
  for (unsigned a = 1; a <= m->imax; a++)
    for (unsigned b = 1; b <= m->jmax; b++)
      if (m->rnew[m->ix(a, b)] > new_jmeanmax) new_jmeanmax = m->rnew[m->ix(a, b)];
  if (m->cycle >= m->time_1) {
    do {
      m->time_1++;
      topmodel_runoff_grid(m, m->time_1);
      if (m->time_step > m->p.max_time_step &&
          new_jmeanmax > (0.2 / (m->jmax * m->imax * DX * DX))) {
        m->cycle = m->time_1 + (m->p.max_time_step / 60);
        m->time_step = m->p.max_time_step;
      }
    } while (m->time_1 < m->cycle);
  }
  calchydrograph_grid(m, m->time_1 - m->cycle);
}

static void catchment_water_input_and_hydrology(hco_model* m, double fdt) {  // :3455-3541
  const double DX = m->DX;
  for (int i = 1; i <= m->p.rfnum; i++)
    m->waterinput += m->j_mean[i] * m->nActualGridCells[i] * DX * DX;
  for (int z = 1; z <= m->totalinputpoints; z++) {
    int i = m->cin_x[z], j = m->cin_y[z];
    int rf = m->rfarea[m->ix(i, j)];
    double amt = (m->j_mean[rf] * m->nActualGridCells[rf]) / (m->cin_counter[rf]) * fdt;
    if (amt > m->p.ERODEFACTOR) amt = m->p.ERODEFACTOR;
    m->H(i, j) += amt;
    if (m->on_grid(i, j)) m->vin_it += amt;
  }
  if (m->cycle >= m->time_1) {
    do {
      m->time_1++;
      topmodel_runoff(m, m->time_1);
      if (m->time_step > m->p.max_time_step) {
        double jmm = 0;
        for (int n = 1; n <= m->p.rfnum; n++)
          if (m->new_j_mean[n] > jmm) jmm = m->new_j_mean[n];
        if (jmm > (0.2 / (m->imax * m->jmax * DX * DX))) {
          m->cycle = m->time_1 + (m->p.max_time_step / 60);
          m->time_step = m->p.max_time_step;
        }
      }
    } while (m->time_1 < m->cycle);
  }
  calchydrograph(m, m->time_1 - m->cycle);
  double jmeanmax = 0;
  for (int n = 1; n <= m->p.rfnum; n++)
    if (m->j_mean[n] > jmeanmax) jmeanmax = m->j_mean[n];
  if (jmeanmax >= m->baseflow) {
    m->baseflow = m->baseflow * 3;
    zero_and_calc_drainage_area(m);
    get_catchment_input_points(m);
  }
  if (m->baseflow > (jmeanmax * 3) && m->baseflow > 0.000001) {
    m->baseflow = jmeanmax * 1.25;
    zero_and_calc_drainage_area(m);
    get_catchment_input_points(m);
  }
}

// ---------------------------------------------------------------------------
// grain store :3874-4171
// ---------------------------------------------------------------------------
static void addGS(hco_model* m, unsigned x, unsigned y);

static void sort_active(hco_model* m, unsigned x, unsigned y) {  // :3874-3947
  if (m->IDX(x, y) == -9999) addGS(m, x, y);
  const int r = m->IDX(x, y);
  const double active = m->p.active;
  double total = 0.0;
  for (unsigned n = 0; n <= G; n++) total += m->GR(r, n);
  if (total > (active * 1.5)) {
    for (unsigned z = 9; z >= 1; z--)
      for (unsigned n = 0; n <= G - 2; n++) m->ST(r, z, n) = m->ST(r, z - 1, n);
    double coeff = active / total;
    for (unsigned n = 1; n <= G - 1; n++)
      if (m->GR(r, n) > 0.0) {
        double amount = coeff * (m->GR(r, n));
        m->ST(r, 0, n - 1) = amount;
        m->GR(r, n) -= amount;
      }
  }
  if (total < (active / 4)) {
    for (unsigned n = 1; n <= G - 1; n++) m->GR(r, n) += m->ST(r, 0, n - 1);
    for (unsigned z = 0; z <= 8; z++)
      for (unsigned n = 0; n <= G - 2; n++) m->ST(r, z, n) = m->ST(r, z + 1, n);
    for (unsigned n = 1; n <= G - 1; n++) m->ST(r, 9, n - 1) = active * m->p.dprop[n];
  }
}

static void addGS(hco_model* m, unsigned x, unsigned y) {  // :3949-3983
  // rows 0 .. N2/LIMIT - 1 exist; past the second last, the cell gets the
  // last row as scratch (no write outside the arrays) and the run stops
  HCO_PRAGMA(omp critical(hco_addGS)) if ((size_t)m->grain_array_tot + 2 >= m->grain.size() / 11) {
    m->grain_full = true;
    m->IDX(x, y) = (int32_t)(m->grain.size() / 11) - 1;
  } else {
    const double active = m->p.active;
    m->grain_array_tot++;
    const int r = m->grain_array_tot;
    m->IDX(x, y) = r;
    m->GR(r, 0) = 0;
    for (unsigned n = 1; n <= G - 1; n++) m->GR(r, n) = active * m->p.dprop[n];
    m->GR(r, G) = 0;
    for (unsigned z = 0; z <= 9; z++) {
      for (unsigned n2 = 0; n2 <= G - 2; n2++) m->ST(r, z, n2) = (active)*m->p.dprop[n2 + 1];
      if (m->E(x, y) - (active * (z + 1)) < (m->bedrock[m->ix(x, y)] - active))
        for (unsigned q = 0; q <= G - 2; q++) m->ST(r, z, q) = 0;
    }
    sort_active(m, x, y);
  }
}

static double sand_fraction(hco_model* m, int r) {  // :3985-4009
  double at = 0, st = 0;
  for (unsigned n = 1; n <= G; n++) at += (m->GR(r, n));
  for (unsigned n = 1; n <= 2; n++) st += (m->GR(r, n));
  if (at < 0.0001) return 0.0;
  return st / at;
}

static double mean_ws_elev(hco_model* m, unsigned x, unsigned y) {  // :4011-4036
  double et = 0;
  int c = 0;
  for (int dir = 1; dir <= 8; dir++) {
    unsigned x2 = x + kDX[dir], y2 = y + kDY[dir];
    if (m->H(x2, y2) > m->p.water_depth_erosion_threshold) {
      et += m->H(x2, y2) + m->E(x2, y2);
      c++;
    }
  }
  if (c > 0) {
    et /= c;
    return et;
  }
  return 0;
}

static double d50(hco_model* m, int r) {  // :4038-4075
  double at = 0, Dfifty = 0, mx = 0, mn = 0;
  double cum[20] = {0};
  for (unsigned n = 1; n <= G; n++) {
    at += (m->GR(r, n));
    cum[n] += at;
  }
  int i = 1;
  while (cum[i] < (at * 0.5) && i <= 9) i++;
  if (i >= 1 && i <= 9) {
    unsigned lo = (i == 1) ? 1 : i - 1;
    mn = std::log(m->Dsize(lo));
    mx = std::log(m->Dsize(i));
  }
  Dfifty = std::exp(mx - ((mx - mn) * ((cum[i] - (at * 0.5)) / (cum[i] - cum[i - 1]))));
  if (at < 0.0000001) Dfifty = 0;
  return Dfifty;
}

static void slide_GS(hco_model* m, unsigned x, unsigned y, double amount, unsigned x2,
                     unsigned y2) {  // :4077-4171
  double total = 0;
  const double* dprop = m->p.dprop;
  if (m->IDX(x, y) != -9999 && m->IDX(x2, y2) != -9999) {
    const int a = m->IDX(x, y), b = m->IDX(x2, y2);
    for (unsigned n = 1; n <= G - 1; n++)
      if (m->GR(a, n) > 0) total += m->GR(a, n);
    if (amount > total) {
      for (unsigned n = 1; n <= G - 1; n++) m->GR(b, n) += (amount - total) * dprop[n];
      amount = total;
    }
    if (total > 0) {
      for (unsigned n = 1; n <= G - 1; n++) {
        double t = amount * (m->GR(a, n) / total);
        m->GR(b, n) += t;
        m->GR(a, n) -= t;
        if (m->GR(a, n) < 0) m->GR(a, n) = 0;
      }
    }
    sort_active(m, x, y);
    sort_active(m, x2, y2);
    return;
  }
  if (m->IDX(x, y) == -9999 && m->IDX(x2, y2) != -9999) {
    const int b = m->IDX(x2, y2);
    for (unsigned n = 1; n <= G - 1; n++) m->GR(b, n) += (amount)*dprop[n];
    sort_active(m, x2, y2);
    return;
  }
  if (m->IDX(x, y) != -9999 && m->IDX(x2, y2) == -9999) {
    addGS(m, x2, y2);
    const int a = m->IDX(x, y), b = m->IDX(x2, y2);
    if (amount > m->p.active) {
      for (unsigned n = 1; n <= G - 1; n++) m->GR(b, n) += amount * dprop[n];
      amount = m->p.active;
    }
    for (unsigned n = 1; n <= G - 1; n++)
      if (m->GR(a, n) > 0) total += m->GR(a, n);
    for (unsigned n = 1; n <= G - 1; n++) {
      if (total > 0) {
        m->GR(b, n) += amount * (m->GR(a, n) / total);
        if (m->GR(a, n) > 0.0001) m->GR(a, n) -= amount * (m->GR(a, n) / total);
        if (m->GR(a, n) < 0) m->GR(a, n) = 0;
      }
    }
    sort_active(m, x, y);
    sort_active(m, x2, y2);
    return;
  }
}

// ---------------------------------------------------------------------------
// water inputs :3301-3452, :2027-2039
// ---------------------------------------------------------------------------
static void reach_water_and_sediment_input(hco_model* m) {  // :3301-3452
  const double fdt = hco_get_flow_timestep(m);
  const double DX = m->DX;
  const int rdt = m->p.reach_input_data_timestep;
  const int div = m->p.div_inputs;
  const double thr = m->p.water_depth_erosion_threshold;
  if (m->p.reach_mode && !m->p.hydro_only) {
    for (int n = 0; n <= m->p.number_of_points - 1; n++) {
      unsigned x = m->p.inpoints[n][0], y = m->p.inpoints[n][1];
      double adding_factor = 1, added_tot = 0;
      if (m->H(x, y) > thr) {
        const std::vector<float>& row = m->reach[n][(int)(m->cycle / rdt)];
        for (int tn = 5; tn <= (int)G + 3; tn++)
          added_tot += (std::abs(row[tn])) / div / (DX * DX) / (rdt * 60) * m->time_step;
        if (added_tot / m->p.number_of_points > m->p.ERODEFACTOR * 0.75)
          adding_factor = (m->p.ERODEFACTOR * 0.75) / (added_tot / m->p.number_of_points);
        if (m->IDX(x, y) == -9999) addGS(m, x, y);
        for (int tn = 5; tn <= (int)G + 3; tn++) {
          double amt = adding_factor * (std::abs(row[tn])) / div / (DX * DX) / (rdt * 60) *
                       m->time_step;
          if (m->p.isSuspended[tn - 4]) {
            m->Vsusptot[m->ix(x, y)] += amt;
          } else {
            m->GR(m->IDX(x, y), tn - 4) += amt;
            m->E(x, y) += amt;
          }
        }
      }
    }
  }
  for (int n = 0; n <= m->p.number_of_points - 1 && m->p.reach_mode; n++) {
    unsigned x = m->p.inpoints[n][0], y = m->p.inpoints[n][1];
    int r = (int)(m->cycle / rdt);
    double i1 = m->reach[n][r][1];
    double i2 = m->reach[n][r + 1][1];
    double prop = (((r + 1) * rdt) - m->cycle) / rdt;
    double input = i1 + ((i2 - i1) * (1 - prop));
    m->waterinput += (input / div);
    const double add = (input / div) / (DX * DX) * fdt;
    m->H(x, y) += add;
    if (m->on_grid(x, y)) m->vin_it += add;
  }
}

// ---------------------------------------------------------------------------
// flow_route :3063-3247
// ---------------------------------------------------------------------------
extern "C" void hco_flow_route(hco_model* m) {
  const double dt = hco_get_flow_timestep(m);
  const unsigned imax = m->imax, jmax = m->jmax;
  const double DX = m->DX, g = kGravity, thr = m->p.hflow_threshold;
  const double es = m->p.edgeslope, fl = m->p.froude_limit;
  const bool susp = m->p.isSuspended[1] != 0;
  double* E = m->elev.data();
  double* Hd = m->water_depth.data();
  double* V = m->Vsusptot.data();
  const size_t W = m->W;
  HCO_PRAGMA(omp parallel for schedule(static))
  for (unsigned y = 1; y <= jmax; y++) {
    int inc = 1;
    while (m->DS(y, inc) > 0) {
      unsigned x = m->DS(y, inc);
      inc++;
      const size_t c = x * W + y, cx = c - W, cy = c - 1;
      if (!(E[c] > -9999)) continue;
      double n = m->mannings;
      if (m->p.spatially_var_mannings) n = m->spat_var_mannings[c];
#ifndef HCO_OPENMP
      m->mannings = n;  // the reference keeps it in a member
#endif
      // x face, between rows x-1 and x
      if ((Hd[c] > 0 || Hd[cx] > 0) && E[cx] > -9999) {
        double hflow = std::max(E[c] + Hd[c], E[cx] + Hd[cx]) - std::max(E[cx], E[c]);
        double& q = m->qx[c];
        if (hflow > thr) {
          double slope = (((E[cx] + Hd[cx])) - (E[c] + Hd[c])) / DX;
          if (x == imax) slope = es;
          if (x <= 2) slope = 0 - es;
          q = ((q - (g * hflow * dt * slope)) /
               (1 + g * hflow * dt * (n * n) * std::abs(q) / std::pow(hflow, 3.0)));
          if (q > 0 && (q / hflow) / std::sqrt(g * hflow) > fl) q = hflow * (std::sqrt(g * hflow) * fl);
          if (q < 0 && std::abs(q / hflow) / std::sqrt(g * hflow) > fl)
            q = 0 - (hflow * (std::sqrt(g * hflow) * fl));
          if (q > 0 && (q * dt / DX) > (Hd[c] / 4)) q = ((Hd[c] * DX) / 5) / dt;
          if (q < 0 && std::abs(q * dt / DX) > (Hd[cx] / 4)) q = 0 - ((Hd[cx] * DX) / 5) / dt;
          if (susp) {
            double& qs = m->qxs[c];
            if (q > 0) qs = q * (V[c] / Hd[c]);
            if (q < 0) qs = q * (V[cx] / Hd[cx]);
            if (qs > 0 && qs * dt > (V[c] * DX) / 4) qs = ((V[c] * DX) / 5) / dt;
            if (qs < 0 && std::abs(qs * dt) > (V[cx] * DX) / 4) qs = 0 - ((V[cx] * DX) / 5) / dt;
          }
          if (q > 0) m->VD(x, y, 7) = q / hflow;
          if (q < 0) m->VD(x - 1, y, 3) = (0 - q) / hflow;
        } else {
          q = 0;
          m->qxs[c] = 0;
        }
      }
      // y face, between columns y-1 and y
      if ((Hd[c] > 0 || Hd[cy] > 0) && E[cy] > -9999) {
        double hflow = std::max(E[c] + Hd[c], E[cy] + Hd[cy]) - std::max(E[c], E[cy]);
        double& q = m->qy[c];
        if (hflow > thr) {
          double slope = (((E[cy] + Hd[cy])) - (E[c] + Hd[c])) / DX;
          if (y == jmax) slope = es;
          if (y <= 2) slope = 0 - es;
          q = ((q - (g * hflow * dt * slope)) /
               (1 + g * hflow * dt * (n * n) * std::abs(q) / std::pow(hflow, 3.0)));
          if (q > 0 && (q / hflow) / std::sqrt(g * hflow) > fl) q = hflow * (std::sqrt(g * hflow) * fl);
          if (q < 0 && std::abs(q / hflow) / std::sqrt(g * hflow) > fl)
            q = 0 - (hflow * (std::sqrt(g * hflow) * fl));
          if (q > 0 && (q * dt / DX) > (Hd[c] / 4)) q = ((Hd[c] * DX) / 5) / dt;
          if (q < 0 && std::abs(q * dt / DX) > (Hd[cy] / 4)) q = 0 - ((Hd[cy] * DX) / 5) / dt;
          if (susp) {
            double& qs = m->qys[c];
            if (q > 0) qs = q * (V[c] / Hd[c]);
            if (q < 0) qs = q * (V[cy] / Hd[cy]);
            if (qs > 0 && qs * dt > (V[c] * DX) / 4) qs = ((V[c] * DX) / 5) / dt;
            if (qs < 0 && std::abs(qs * dt) > (V[cy] * DX) / 4) qs = 0 - ((V[cy] * DX) / 5) / dt;
          }
          if (q > 0) m->VD(x, y, 1) = q / hflow;
          if (q < 0) m->VD(x, y - 1, 5) = (0 - q) / hflow;
        } else {
          q = 0;
          m->qys[c] = 0;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// depth_update :3259-3299
// ---------------------------------------------------------------------------
extern "C" void hco_depth_update(hco_model* m) {
  const double dt = hco_get_flow_timestep(m);
  const unsigned jmax = m->jmax;
  const double DX = m->DX;
  const bool susp = m->p.isSuspended[1] != 0;
  const size_t W = m->W;
  double* Hd = m->water_depth.data();
  m->maxdepth = 0;
  double l_max = m->maxdepth;
  // The ledger (not part of the reference): a face between a listed cell
  // and one outside down_scan changes only the listed cell's depth, so the
  // water crossing it appears or vanishes; `edge` sums it, in the same
  // expression form as the update.
  std::vector<uint8_t>& L = m->listed;
  L.assign(m->N2, 0);
  for (unsigned y = 1; y <= jmax; y++)
    for (int inc = 1; m->DS(y, inc) > 0; inc++) L[m->DS(y, inc) * W + y] = 1;
  double lost = 0, edge = 0;
  HCO_PRAGMA(omp parallel for reduction(max : l_max) reduction(+ : lost, edge) schedule(static))
  for (unsigned y = 1; y <= jmax; y++) {
    int inc = 1;
    double tmax = 0;
    while (m->DS(y, inc) > 0) {
      unsigned x = m->DS(y, inc);
      inc++;
      const size_t c = x * W + y;
      if (!L[c - W] || !L[c + W] || !L[c - 1] || !L[c + 1]) {
        const double ux1 = L[c + W] ? 0.0 : m->qx[c + W], ux0 = L[c - W] ? 0.0 : m->qx[c];
        const double uy1 = L[c + 1] ? 0.0 : m->qy[c + 1], uy0 = L[c - 1] ? 0.0 : m->qy[c];
        edge += dt * (ux1 - ux0 + uy1 - uy0) / DX;
      }
      Hd[c] += dt * (m->qx[c + W] - m->qx[c] + m->qy[c + 1] - m->qy[c]) / DX;
      if (susp)
        m->Vsusptot[c] += dt * (m->qxs[c + W] - m->qxs[c] + m->qys[c + 1] - m->qys[c]) / DX;
      if (Hd[c] > 0) {
        if (m->elev[c] == -9999) {
          lost += Hd[c];
          Hd[c] = 0;
        }
        if (Hd[c] > tmax) tmax = Hd[c];
      }
    }
    if (tmax > l_max) l_max = tmax;
  }
  m->maxdepth = l_max;
  m->vlost_it += lost;
  m->vmask_it += edge;
}

// ---------------------------------------------------------------------------
// scan_area :3821-3849
// ---------------------------------------------------------------------------
extern "C" void hco_scan_area(hco_model* m) {
  const unsigned imax = m->imax, jmax = m->jmax;
  HCO_PRAGMA(omp parallel for schedule(static))
  for (unsigned j = 1; j <= jmax; j++) {
    int inc = 1;
    for (unsigned i = 1; i <= imax; i++) {
      m->DS(j, i) = 0;
      if (m->H(i, j) > 0 || m->H(i, j - 1) > 0 || m->H(i, j + 1) > 0 || m->H(i - 1, j) > 0 ||
          m->H(i - 1, j - 1) > 0 || m->H(i - 1, j + 1) > 0 || m->H(i + 1, j - 1) > 0 ||
          m->H(i + 1, j + 1) > 0 || m->H(i + 1, j) > 0) {
        m->DS(j, inc) = i;
        inc++;
      }
    }
  }
  // the ledger's volume after depth_update (not part of the reference)
  double vol = 0;
  HCO_PRAGMA(omp parallel for reduction(+ : vol) schedule(static))
  for (unsigned i = 1; i <= imax; i++)
    for (unsigned j = 1; j <= jmax; j++) vol += m->H(i, j);
  m->vol_scan = vol;
  m->vol_scan_counter = m->counter;
}

// ---------------------------------------------------------------------------
// water_flux_out :3005-3047
// ---------------------------------------------------------------------------
extern "C" void hco_water_flux_out(hco_model* m) {
  const double fdt = m->time_step, thr = m->p.water_depth_erosion_threshold, DX = m->DX;
  const unsigned imax = m->imax, jmax = m->jmax;
  m->temptot = 0;
  auto clamp = [&](unsigned i, unsigned j) {
    double& h = m->H(i, j);
    if (h > thr) {
      m->temptot += (h - thr) * DX * DX / fdt;
      m->vout_it += h - thr;
      h = thr;
    }
  };
  for (unsigned i = 1; i <= imax; i++) {
    clamp(i, jmax);
    clamp(i, 1);
  }
  for (unsigned j = 1; j <= jmax; j++) {
    clamp(1, j);
    clamp(imax, j);
  }
  m->waterOut = m->temptot;
}

// ---------------------------------------------------------------------------
// erode :4211-4845
// ---------------------------------------------------------------------------
extern "C" double hco_erode(hco_model* m, double mult_factor) {
  const double rho = 1000.0, g = kGravity, DX = m->DX;
  const unsigned imax = m->imax, jmax = m->jmax;
  const double thr = m->p.water_depth_erosion_threshold;
  const double ERODEFACTOR = m->p.ERODEFACTOR;
  const double* dprop = m->p.dprop;
  const int* isSusp = m->p.isSuspended;
  const bool wilcock = m->p.wilcock != 0, einstein = m->p.einstein != 0;
  double tempbmax = 0;
  float gtot2[20] = {};

  m->time_step = m->time_step * 1.5;

  do {
    tempbmax = 0;
    HCO_PRAGMA(omp parallel for reduction(max : tempbmax) schedule(static))
    for (unsigned y = 1; y < jmax; ++y) {
      int inc = 1;
      while (m->DS(y, inc) > 0) {
        unsigned x = m->DS(y, inc);
        inc++;
        const size_t c = m->ix(x, y);
        m->Vel[c] = 0;
        m->Tau[c] = 0;
        for (unsigned n = 0; n < G; n++) {
          m->S4(m->sr, x, y, n) = 0;
          m->S4(m->sl, x, y, n) = 0;
          m->S4(m->su, x, y, n) = 0;
          m->S4(m->sd, x, y, n) = 0;
        }
        m->ss[c] = 0;
        if (m->H(x, y) > thr) {
          double temptot2 = 0, veltot = 0, vel = 0, qtot = 0, tau = 0, slopetot = 0;
          double tempdir[11] = {}, temp_dist[11] = {};
          double n_man = m->mannings;
          if (m->p.spatially_var_mannings) n_man = m->spat_var_mannings[c];
#ifndef HCO_OPENMP
          m->mannings = n_man;
#endif
          if (m->IDX(x, y) == -9999) addGS(m, x, y);
          for (int p = 1; p <= 8; p += 2) {
            unsigned x2 = x + kDX[p], y2 = y + kDY[p];
            if (m->H(x2, y2) > thr) {
              if (m->EDGE(x, y) > m->EDGE(x2, y2)) temptot2 += (m->EDGE(x, y) - m->EDGE(x2, y2));
              if (m->VD(x, y, p) > 0) {
                vel = m->VD(x, y, p);
                if (vel > m->p.max_vel) vel = m->p.max_vel;
                tempdir[p] = vel * vel;
                veltot += tempdir[p];
                qtot += (vel * vel);
                slopetot += ((m->E(x, y) - m->E(x2, y2)) / DX) * vel;
              }
            }
          }
          if (qtot > 0) {
            vel = (std::sqrt(qtot));
            m->Vel[c] = vel;
            if (vel > m->p.max_vel) vel = m->p.max_vel;
            double ci = g * (n_man * n_man) * std::pow(m->H(x, y), -0.33);
            if (slopetot > 0) slopetot = 0;
            tau = 1000 * ci * vel * vel * (1 + (1 * (slopetot / vel)));
            m->Tau[c] = tau;
          }
          if (tau > 0) {
            const int r = m->IDX(x, y);
            double d_50 = 0, Fs = 0, Di = 0, graintot = 0;
            if (wilcock) {
              d_50 = d50(m, r);
              if (d_50 < m->Dsize(1)) d_50 = m->Dsize(1);
              Fs = sand_fraction(m, r);
              for (unsigned n = 1; n <= G; n++) graintot += (m->GR(r, n));
            }
            double temptot1 = 0;
            for (unsigned n = 1; n <= G - 1; n++) {
              Di = m->Dsize(n);
              if (wilcock) {
                double tau_ri = (0.021 + (0.015 * std::exp(-20 * Fs))) * (rho * g * d_50) *
                                std::pow((Di / d_50), (0.67 / (1 + std::exp(1.5 - (Di / d_50)))));
                double U_star = std::pow(tau / rho, 0.5);
                double Fi = m->GR(r, n) / graintot;
                double Wi_star;
                if ((tau / tau_ri) < 1.35)
                  Wi_star = 0.002 * std::pow(tau / tau_ri, 7.5);
                else
                  Wi_star = 14 * std::pow(1 - (0.894 / std::pow(tau / tau_ri, 0.5)), 4.5);
                temp_dist[n] = mult_factor * m->time_step *
                               ((Fi * (U_star * U_star * U_star)) / ((2.65 - 1) * g)) * Wi_star / DX;
              }
              if (einstein) {
                temp_dist[n] = mult_factor * m->time_step *
                               (40 * std::pow((1 / (((2650 - 1000) * Di) / (tau / g))), 3.0)) /
                               std::sqrt(1000 / ((2250 - 1000) * g * (Di * Di * Di))) / DX;
              }
              if (temp_dist[n] > m->GR(r, n)) temp_dist[n] = m->GR(r, n);
              if (isSusp[n] && n == 1) {
                if ((temp_dist[n] + m->Vsusptot[c]) / m->H(x, y) > m->p.Csuspmax)
                  temp_dist[n] = (m->H(x, y) * m->p.Csuspmax) - m->Vsusptot[c];
              }
              if (temp_dist[n] < 0) temp_dist[n] = 0;
              temptot1 += temp_dist[n];
            }
            if (m->E(x, y) - temptot1 <= m->bedrock[c]) {
              double elevdiff = m->E(x, y) - m->bedrock[c];
              double temptot3 = temptot1;
              temptot1 = 0;
              for (unsigned n = 1; n <= G - 1; n++) {
                if (m->E(x, y) <= m->bedrock[c]) {
                  temp_dist[n] = 0;
                } else {
                  temp_dist[n] = elevdiff * (temp_dist[n] / temptot3);
                  if (temp_dist[n] < 0) temp_dist[n] = 0;
                }
                temptot1 += temp_dist[n];
              }
              if (tau > m->p.bedrock_erosion_threshold) {
                double amount = std::pow(m->p.bedrock_erosion_rate * tau, 1.5) * m->time_step *
                                mult_factor * 0.000000317;
                m->bedrock[c] -= amount;
                for (unsigned n2 = 1; n2 <= G - 1; n2++) m->GR(r, n2) += amount * dprop[n2];
              }
            }
            if (m->VEG(x, y, 1) > 0 && tau > m->p.vegTauCrit) {
              m->VEG(x, y, 1) -= mult_factor * m->time_step * std::pow(tau - m->p.vegTauCrit, 0.5) * 0.00001;
              if (m->VEG(x, y, 1) < 0) m->VEG(x, y, 1) = 0;
            }
            if (m->VEG(x, y, 1) > 0.25) {
              if (m->E(x, y) - temptot1 <= m->VEG(x, y, 0)) {
                double elevdiff = m->E(x, y) - m->VEG(x, y, 0);
                if (elevdiff < 0) elevdiff = 0;
                double temptot3 = temptot1;
                temptot1 = 0;
                for (unsigned n = 1; n <= G - 1; n++) {
                  temp_dist[n] = elevdiff * (temp_dist[n] / temptot3);
                  if (m->E(x, y) <= m->VEG(x, y, 0)) temp_dist[n] = 0;
                  temptot1 += temp_dist[n];
                }
                if (temptot1 < 0) temptot1 = 0;
              }
            }
            if (temptot1 > tempbmax) tempbmax = temptot1;
            if (temptot1 > 0) {
              for (int p = 1; p <= 8; p += 2) {
                unsigned x2 = x + kDX[p], y2 = y + kDY[p];
                if (m->H(x2, y2) > thr) {
                  if (m->IDX(x2, y2) == -9999) addGS(m, x2, y2);
                  double factor = 0;
                  if (m->VD(x, y, p) > 0) factor += 0.75 * tempdir[p] / veltot;
                  if (m->EDGE(x, y) > m->EDGE(x2, y2))
                    factor += 0.25 * ((m->EDGE(x, y) - m->EDGE(x2, y2)) / temptot2);
                  for (unsigned n = 1; n <= G - 1; n++) {
                    if (temp_dist[n] > 0) {
                      if (n == 1 && isSusp[n]) {
                        m->ss[c] = temp_dist[n];
                      } else {
                        switch (p) {
                          case 1: m->S4(m->su, x, y, n) = temp_dist[n] * factor; break;
                          case 3: m->S4(m->sr, x, y, n) = temp_dist[n] * factor; break;
                          case 5: m->S4(m->sd, x, y, n) = temp_dist[n] * factor; break;
                          case 7: m->S4(m->sl, x, y, n) = temp_dist[n] * factor; break;
                        }
                      }
                    }
                  }
                }
              }
            }
          }
        }
      }
    }
    if (tempbmax > ERODEFACTOR) m->time_step *= (ERODEFACTOR / tempbmax) * 0.5;
  } while (tempbmax > ERODEFACTOR);

  std::vector<double> erodetot(m->N2, 0.0), erodetot3(m->N2, 0.0);
  const double lc = m->p.lateral_constant, cle = m->p.chann_lateral_erosion;
  const double vlr = m->p.veg_lat_restriction;

  HCO_PRAGMA(omp parallel for schedule(static))
  for (unsigned y = 2; y < jmax; ++y) {
    int inc = 1;
    while (m->DS(y, inc) > 0) {
      unsigned x = m->DS(y, inc);
      inc++;
      const size_t c = m->ix(x, y);
      if (m->H(x, y) > thr && x < imax && x > 1) {
        if (m->IDX(x, y) == -9999) addGS(m, x, y);
        const int r = m->IDX(x, y);
        for (unsigned n = 1; n <= G - 1; n++) {
          if (n == 1 && isSusp[n]) {
            m->Vsusptot[c] += m->ss[c];
            m->GR(r, n) -= m->ss[c];
            erodetot[c] -= m->ss[c];
            if (!m->inputpointsarray[c]) {
              double coeff = (m->p.fallVelocity[n] * m->time_step) / m->H(x, y);
              if (coeff > 1) coeff = 1;
              double Vpdrop = coeff * m->Vsusptot[c];
              if (Vpdrop > 0.001) Vpdrop = 0.001;
              m->GR(r, n) += Vpdrop;
              erodetot[c] += Vpdrop;
              m->Vsusptot[c] -= Vpdrop;
            }
          } else {
            double val1 = (m->S4(m->su, x, y, n) + m->S4(m->sr, x, y, n) + m->S4(m->sd, x, y, n) +
                           m->S4(m->sl, x, y, n));
            double val2 = (m->S4(m->su, x, y + 1, n) + m->S4(m->sd, x, y - 1, n) +
                           m->S4(m->sl, x + 1, y, n) + m->S4(m->sr, x - 1, y, n));
            m->GR(r, n) += val2 - val1;
            erodetot[c] += val2 - val1;
            erodetot3[c] += val1;
          }
        }
        m->E(x, y) += erodetot[c];
        if (erodetot[c] < 0) sort_active(m, x, y);
        if (erodetot3[c] > 0) {
          double elev_update = 0;
          if (m->E(x - 1, y) > m->E(x, y) && x > 2) {
            double amt = 0;
            if (m->H(x - 1, y) < thr)
              amt = mult_factor * lc * m->Tau[c] * m->EDGE(x - 1, y) * m->time_step / DX;
            else
              amt = cle * erodetot3[c] * (m->E(x - 1, y) - m->E(x, y)) / DX * 0.1;
            if (amt > 0) {
              amt *= 1 - (m->VEG(x - 1, y, 1) * (1 - vlr));
              if ((m->E(x - 1, y) - amt) < m->bedrock[m->ix(x - 1, y)] || x - 1 == 1) amt = 0;
              if (amt > ERODEFACTOR * 0.1) amt = ERODEFACTOR * 0.1;
              elev_update += amt;
              m->E(x - 1, y) -= amt;
              slide_GS(m, x - 1, y, amt, x, y);
            }
          }
          if (m->E(x + 1, y) > m->E(x, y) && x < imax - 1) {
            double amt = 0;
            if (m->H(x + 1, y) < thr)
              amt = mult_factor * lc * m->Tau[c] * m->EDGE(x + 1, y) * m->time_step / DX;
            else
              amt = cle * erodetot3[c] * (m->E(x + 1, y) - m->E(x, y)) / DX * 0.1;
            if (amt > 0) {
              amt *= 1 - (m->VEG(x + 1, y, 1) * (1 - vlr));
              if ((m->E(x + 1, y) - amt) < m->bedrock[m->ix(x + 1, y)] || x + 1 == imax) amt = 0;
              if (amt > ERODEFACTOR * 0.1) amt = ERODEFACTOR * 0.1;
              elev_update += amt;
              m->E(x + 1, y) -= amt;
              slide_GS(m, x + 1, y, amt, x, y);
            }
          }
          m->E(x, y) += elev_update;
        }
      }
    }
  }

  HCO_PRAGMA(omp parallel for schedule(static))
  for (unsigned y = 2; y < jmax; ++y) {
    int inc = 1;
    while (m->DS(y, inc) > 0) {
      unsigned x = m->DS(y, inc);
      inc++;
      const size_t c = m->ix(x, y);
      if (erodetot3[c] > 0) {
        double elev_update = 0;
        if (m->E(x, y - 1) > m->E(x, y)) {
          double amt = 0;
          if (m->H(x, y - 1) < thr)
            amt = mult_factor * lc * m->Tau[c] * m->EDGE(x, y - 1) * m->time_step / DX;
          else
            amt = cle * erodetot3[c] * (m->E(x, y - 1) - m->E(x, y)) / DX * 0.1;
          if (amt > 0) {
            amt *= 1 - (m->VEG(x, y - 1, 1) * (1 - vlr));
            if ((m->E(x, y - 1) - amt) < m->bedrock[m->ix(x, y - 1)] || y - 1 == 1) amt = 0;
            if (amt > ERODEFACTOR * 0.1) amt = ERODEFACTOR * 0.1;
            elev_update += amt;
            m->E(x, y - 1) -= amt;
            slide_GS(m, x, y - 1, amt, x, y);
          }
        }
        if (m->E(x, y + 1) > m->E(x, y)) {
          double amt = 0;
          if (m->H(x, y + 1) < thr)
            amt = mult_factor * lc * m->Tau[c] * m->EDGE(x, y + 1) * m->time_step / DX;
          else
            amt = cle * erodetot3[c] * (m->E(x, y + 1) - m->E(x, y)) / DX * 0.1;
          if (amt > 0) {
            amt *= 1 - (m->VEG(x, y + 1, 1) * (1 - vlr));
            if ((m->E(x, y + 1) - amt) < m->bedrock[m->ix(x, y + 1)] || y + 1 == jmax) amt = 0;
            if (amt > ERODEFACTOR * 0.1) amt = ERODEFACTOR * 0.1;
            elev_update += amt;
            m->E(x, y + 1) -= amt;
            slide_GS(m, x, y + 1, amt, x, y);
          }
        }
        m->E(x, y) += elev_update;
      }
    }
  }

  // sediment leaving the four edges, accumulated in float as the reference does
  HCO_PRAGMA(omp parallel for reduction(+ : gtot2[:20]))
  for (unsigned y = 2; y < jmax; y++) {
    if (m->H(imax, y) > thr || m->Vsusptot[m->ix(imax, y)] > 0) {
      for (unsigned n = 1; n <= G - 1; n++) {
        if (isSusp[n]) {
          gtot2[n] += m->Vsusptot[m->ix(imax, y)];
          m->Vsusptot[m->ix(imax, y)] = 0;
        } else {
          gtot2[n] += m->S4(m->sr, imax - 1, y, n);
        }
      }
    }
    if (m->H(1, y) > thr || m->Vsusptot[m->ix(1, y)] > 0) {
      for (unsigned n = 1; n <= G - 1; n++) {
        if (isSusp[n]) {
          gtot2[n] += m->Vsusptot[m->ix(1, y)];
          m->Vsusptot[m->ix(1, y)] = 0;
        } else {
          gtot2[n] += m->S4(m->sl, 2, y, n);
        }
      }
    }
  }
  HCO_PRAGMA(omp parallel for reduction(+ : gtot2[:20]))
  for (unsigned x = 2; x < imax; x++) {
    if (m->H(x, jmax) > thr || m->Vsusptot[m->ix(x, jmax)] > 0) {
      for (unsigned n = 1; n <= G - 1; n++) {
        if (isSusp[n]) {
          gtot2[n] += m->Vsusptot[m->ix(x, jmax)];
          m->Vsusptot[m->ix(x, jmax)] = 0;
        } else {
          gtot2[n] += m->S4(m->sd, x, jmax - 1, n);
        }
      }
    }
    if (m->H(x, 1) > thr || m->Vsusptot[m->ix(x, 1)] > 0) {
      for (unsigned n = 1; n <= G - 1; n++) {
        if (isSusp[n]) {
          gtot2[n] += m->Vsusptot[m->ix(x, 1)];
          m->Vsusptot[m->ix(x, 1)] = 0;
        } else {
          gtot2[n] += m->S4(m->su, x, 2, n);
        }
      }
    }
  }
  m->sediQ = 0;
  for (unsigned n = 1; n <= G; n++) {
    m->sediQ += gtot2[n] * DX * DX;
    m->globalsediq += gtot2[n] * DX * DX;
    m->sum_grain[n] += gtot2[n] * DX * DX;
  }
  m->tempbmax = tempbmax;
  return tempbmax;
}

// ---------------------------------------------------------------------------
// lateral_channel_erode :4850-5291  (square grids: the reference indexes the
// edge arrays with x < jmax+1 and y < imax+1)
// ---------------------------------------------------------------------------
namespace {
struct Grid {
  std::vector<double> v;
  size_t w;
  Grid(size_t a, size_t b, double init) : v(a * b, init), w(b) {}
  double& operator()(size_t i, size_t j) { return v[i * w + j]; }
};
struct IGrid {
  std::vector<int> v;
  size_t w;
  IGrid(size_t a, size_t b) : v(a * b, 0), w(b) {}
  int& operator()(size_t i, size_t j) { return v[i * w + j]; }
};

inline bool edge_neighbour_counts(hco_model* m, Grid& wd2, unsigned x, unsigned y, int dir,
                                  double mft) {
  // Whether neighbour dir of (x,y) joins the edge mean (:5061-5196): Manhattan
  // neighbours need a wet diagonal beside them, diagonals a dry link cell.
  const int dx = kDX[dir], dy = kDY[dir];
  if ((std::abs(dx) + std::abs(dy)) != 2) {
    if (dx == 1 && dy == 0 && (wd2(x + 1, y - 1) > mft || wd2(x + 1, y + 1) > mft)) return true;
    if (dx == 0 && dy == 1 && (wd2(x + 1, y + 1) > mft || wd2(x - 1, y + 1) > mft)) return true;
    if (dx == -1 && dy == 0 && (wd2(x - 1, y - 1) > mft || wd2(x - 1, y + 1) > mft)) return true;
    if (dx == 0 && dy == -1 && (wd2(x - 1, y - 1) > mft || wd2(x + 1, y - 1) > mft)) return true;
  } else {
    if (dx == -1 && dy == -1 && (wd2(x, y - 1) < mft || wd2(x - 1, y) < mft)) return true;
    if (dx == 1 && dy == -1 && (wd2(x, y - 1) < mft || wd2(x + 1, y) < mft)) return true;
    if (dx == 1 && dy == 1 && (wd2(x + 1, y) < mft || wd2(x, y + 1) < mft)) return true;
    if (dx == -1 && dy == 1 && (wd2(x, y + 1) < mft || wd2(x - 1, y) < mft)) return true;
  }
  return false;
}
}  // namespace

extern "C" void hco_lateral_channel_erode(hco_model* m) {
  const unsigned imax = m->imax, jmax = m->jmax;
  if (imax != jmax) return;  // the reference is only defined on square grids
  Grid edge_temp(jmax + 1, imax + 1, 0.0);
  Grid wd2(jmax + 1, imax + 1, 0.0);
  IGrid upscale((jmax + 1) * 2, (imax + 1) * 2);
  IGrid upscale_edge((jmax + 1) * 2, (imax + 1) * 2);
  const double mft = 0.1;

  for (unsigned y = 2; y < jmax; y++) {  // :4863-4890
    int inc = 1;
    while (m->DS(y, inc) > 0) {
      unsigned x = m->DS(y, inc);
      edge_temp(x, y) = 0;
      if (x == 1) x++;
      if (x == jmax) x--;
      inc++;
      if (m->Tau[m->ix(x, y)] > mft) {
        wd2(x, y) = m->Tau[m->ix(x, y)];
        int tc = 0;
        for (int dir = 1; dir <= 8; dir++)
          if (m->Tau[m->ix(x + kDX[dir], y + kDY[dir])] < mft) tc++;
        if (tc > 6) wd2(x, y) = 0;
      }
    }
  }
  for (unsigned y = 2; y < imax; y++) {  // :4894-4939
    for (unsigned x = 2; x < jmax; x++) {
      m->EDGE(x, y) = -9999;
      if (wd2(x, y) < mft) {
        if (wd2(x, y - 1) > mft || wd2(x - 1, y) > mft || wd2(x + 1, y) > mft || wd2(x, y + 1) > mft)
          m->EDGE(x, y) = 0;
        if (wd2(x, y - 1) > mft && wd2(x - 1, y) > mft && wd2(x + 1, y) > mft && wd2(x, y + 1) > mft) {
          m->EDGE(x, y) = -9999;
          m->edge2[m->ex(x, y)] = -9999;
        }
        upscale(x * 2, y * 2) = 0;
        upscale(x * 2, y * 2 - 1) = 0;
        upscale(x * 2 - 1, y * 2) = 0;
        upscale(x * 2 - 1, y * 2 - 1) = 0;
      }
      if (wd2(x, y) >= mft) {
        upscale(x * 2, y * 2) = 1;
        upscale(x * 2, y * 2 - 1) = 1;
        upscale(x * 2 - 1, y * 2) = 1;
        upscale(x * 2 - 1, y * 2 - 1) = 1;
      }
    }
  }
  for (unsigned y = 2; y < imax * 2; y++)  // :4942-4958
    for (unsigned x = 2; x < jmax * 2; x++) {
      upscale_edge(x, y) = 0;
      if (upscale(x, y) == 0)
        if (upscale(x, y - 1) == 1 || upscale(x - 1, y) == 1 || upscale(x + 1, y) == 1 ||
            upscale(x, y + 1) == 1)
          upscale(x, y) = 2;
    }
  for (unsigned y = 2; y < imax * 2; y++)  // :4961-4991
    for (unsigned x = 2; x < jmax * 2; x++)
      if (upscale(x, y) == 2) {
        int wet = 0, dry = 0, ecc = 1;
        for (int dir = 1; dir <= 7; dir += 2) {
          int v = upscale(x + kDX[dir], y + kDY[dir]);
          if (v == 1) wet += 1;
          if (v == 0) dry += 1;
          if (v == 2) ecc += 1;
        }
        if (ecc > 3) dry += ecc - 2;
        upscale_edge(x, y) = wet - dry;
      }
  for (unsigned x = 1; x <= jmax; x++)  // :4994-5009
    for (unsigned y = 1; y <= imax; y++)
      if (m->EDGE(x, y) == 0) {
        m->EDGE(x, y) = (double)(upscale_edge(x * 2, y * 2) + upscale_edge(x * 2, y * 2 - 1) +
                                 upscale_edge(x * 2 - 1, y * 2) + upscale_edge(x * 2 - 1, y * 2 - 1));
        if (m->EDGE(x, y) > 2) m->EDGE(x, y) = 2;
        if (m->EDGE(x, y) < -2) m->EDGE(x, y) = -2;
      }

  const double esp = m->p.edge_smoothing_passes;
  for (int n = 1; n <= esp + m->p.downstream_shift; n++) {  // :5011-5208
    HCO_PRAGMA(omp parallel for schedule(static))
    for (unsigned y = 2; y < imax; y++) {
      int inc = 1;
      while (m->DS(y, inc) > 0) {
        unsigned x = m->DS(y, inc);
        edge_temp(x, y) = 0;
        if (x == 1) x++;
        if (x == jmax) x--;
        if (y == 1) break;
        if (y == imax) break;
        inc++;
        if (m->EDGE(x, y) > -9999) {
          double mean = 0, num = 0;
          mean += m->EDGE(x, y);
          num++;
          for (int dir = 1; dir <= 8; dir++) {
            unsigned x2 = x + kDX[dir], y2 = y + kDY[dir];
            bool take = false;
            if (n > esp && m->EDGE(x2, y2) > -9999 && wd2(x2, y2) < mft &&
                mean_ws_elev(m, x2, y2) > mean_ws_elev(m, x, y))
              take = edge_neighbour_counts(m, wd2, x, y, dir, mft);
            else if (n <= esp && m->EDGE(x2, y2) > -9999 && wd2(x2, y2) < mft)
              take = edge_neighbour_counts(m, wd2, x, y, dir, mft);
            if (take) {
              mean += (m->EDGE(x + kDX[dir], y + kDY[dir]));
              num++;
            }
          }
          if (mean != 0) edge_temp(x, y) = mean / num;
          if (x < 3 || x > (jmax - 3)) edge_temp(x, y) = 0;
          if (y < 3 || y > (imax - 3)) edge_temp(x, y) = 0;
        }
      }
    }
    for (unsigned y = 2; y < imax; y++) {
      int inc = 1;
      while (m->DS(y, inc) > 0) {
        unsigned x = m->DS(y, inc);
        inc++;
        if (m->EDGE(x, y) > -9999) m->EDGE(x, y) = edge_temp(x, y);
      }
    }
  }
  for (unsigned x = 1; x <= jmax; x++)  // :5210-5227
    for (unsigned y = 1; y <= imax; y++) {
      double& e = m->EDGE(x, y);
      if (e > -9999) {
        if (e > 0) e = 0;
        e = 0 - e;
        e = 1 / ((2.131 * std::pow(e, -1.0794)) * m->DX);
      }
      if (m->H(x, y) > m->p.water_depth_erosion_threshold && e == -9999) e = 0;
    }
  double tempdiff = 0;
  do {  // :5229-5288
    for (unsigned y = 2; y < imax; y++) {
      int inc = 1;
      while (m->DS(y, inc) > 0) {
        unsigned x = m->DS(y, inc);
        edge_temp(x, y) = 0;
        if (x == 1) x++;
        if (x == jmax) x--;
        inc++;
        if (wd2(x, y) > mft && m->EDGE(x, y) == -9999) m->EDGE(x, y) = 0;
        if (m->EDGE(x, y) > -9999 && wd2(x, y) > mft) {
          double mean = 0;
          int num = 0;
          for (int dir = 1; dir <= 8; dir += 2) {
            unsigned x2 = x + kDX[dir], y2 = y + kDY[dir];
            if (wd2(x2, y2) > mft && m->EDGE(x2, y2) == -9999) m->EDGE(x2, y2) = 0;
            if (m->EDGE(x2, y2) > -9999) {
              mean += (m->EDGE(x2, y2));
              num++;
            }
          }
          edge_temp(x, y) = mean / num;
        }
      }
    }
    tempdiff = 0;
    for (unsigned y = 2; y < imax; y++) {
      int inc = 1;
      while (m->DS(y, inc) > 0) {
        unsigned x = m->DS(y, inc);
        if (x == 1) x++;
        if (x == jmax) x--;
        inc++;
        if (m->EDGE(x, y) > -9999 && wd2(x, y) > mft) {
          if (std::abs(m->EDGE(x, y) - edge_temp(x, y)) > tempdiff)
            tempdiff = std::abs(m->EDGE(x, y) - edge_temp(x, y));
          m->EDGE(x, y) = edge_temp(x, y);
        }
      }
    }
  } while (tempdiff > m->p.lateral_cross_channel_smoothing);
}

// ---------------------------------------------------------------------------
// in_channel_landsliding :5429-5527
// ---------------------------------------------------------------------------
extern "C" void hco_in_channel_landsliding(hco_model* m) {
  const unsigned imax = m->imax, jmax = m->jmax;
  const double factor = std::tan((m->p.failureangle * (3.141592654 / 180))) * m->DX;
  const double active = m->p.active;
  // neighbour order of the reference's eight tests
  static const int ox[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  static const int oy[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  for (unsigned y = 2; y < jmax; y++) {
    unsigned inc = 1;
    while (m->DS(y, inc) > 0) {
      unsigned x = m->DS(y, inc);
      if (x == imax) x = imax - 1;
      if (x == 1) x = 2;
      inc++;
      double wet_factor = factor;
      const size_t c = m->ix(x, y);
      if (m->elev[c] <= (m->bedrock[c] + active)) wet_factor = 10000;
      for (int k = 0; k < 8; k++) {
        unsigned x2 = x + ox[k], y2 = y + oy[k];
        const bool diag = (ox[k] != 0 && oy[k] != 0);
        double drop = diag ? ((m->elev[c] - m->E(x2, y2)) / 1.41) : (m->elev[c] - m->E(x2, y2));
        if (drop > wet_factor && m->E(x2, y2) > -9999) {
          double diff = diag ? (((m->elev[c] - m->E(x2, y2)) / 1.41) - wet_factor)
                             : ((m->elev[c] - m->E(x2, y2)) - wet_factor);
          if ((m->elev[c] - diff) < (m->bedrock[c] + active))
            diff = (m->elev[c] - (m->bedrock[c] + active));
          m->elev[c] -= diff;
          m->E(x2, y2) += diff;
          slide_GS(m, x, y, diff, x2, y2);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// creep :5293-5427 and global_landsliding :5529-5654 (outside the per-step
// path; run at iteration 1 and on their long intervals)
// ---------------------------------------------------------------------------
extern "C" void hco_creep(hco_model* m, double time) {
  const unsigned imax = m->imax, jmax = m->jmax;
  const double DX = m->DX, root = 7.07, CR = m->p.CREEP_RATE;
  for (unsigned x = 1; x <= imax; x++)
    for (unsigned y = 1; y <= jmax; y++) m->tempcreep[m->ix(x, y)] = 0;
  // neighbour order of the reference's eight tests
  static const int ox[8] = {0, 1, 1, 1, 0, -1, -1, -1};
  static const int oy[8] = {-1, -1, 0, 1, 1, 1, 0, -1};
  for (unsigned x = 2; x < imax; x++)
    for (unsigned y = 2; y < jmax; y++) {
      const size_t c = m->ix(x, y);
      if (m->elev[c] > m->bedrock[c]) {
        for (int k = 0; k < 8; k++) {
          unsigned x2 = x + ox[k], y2 = y + oy[k];
          const bool diag = (ox[k] != 0 && oy[k] != 0);
          if (m->E(x2, y2) < m->elev[c] && m->E(x2, y2) > -9999) {
            double temp = diag ? ((m->elev[c] - m->E(x2, y2)) / root) * CR * time / root
                               : ((m->elev[c] - m->E(x2, y2)) / DX) * CR * time / DX;
            if ((m->elev[c] - temp) < m->bedrock[c]) temp = m->elev[c] - m->bedrock[c];
            if (temp < 0) temp = 0;
            m->tempcreep[c] -= temp;
            m->tempcreep[m->ix(x2, y2)] += temp;
            if (m->IDX(x, y) != -9999) slide_GS(m, x, y, temp, x2, y2);
          }
        }
      }
    }
  for (unsigned x = 1; x <= imax; x++)
    for (unsigned y = 1; y <= jmax; y++) m->E(x, y) += m->tempcreep[m->ix(x, y)];
}

extern "C" void hco_global_landsliding(hco_model* m) {
  const unsigned imax = m->imax, jmax = m->jmax;
  const double factor = std::tan((m->p.failureangle * (3.141592654 / 180))) * m->DX;
  const double active = m->p.active, EF = m->p.ERODEFACTOR;
  static const int ox[8] = {1, 0, -1, -1, -1, 0, 1, 1};
  static const int oy[8] = {1, 1, 1, 0, -1, -1, -1, 0};
  unsigned inc = 0;
  double total = 0;
  do {
    total = 0;
    inc++;
    for (unsigned x = 2; x < imax; x++)
      for (unsigned y = 2; y < jmax; y++) {
        const size_t c = m->ix(x, y);
        double wet_factor = factor;
        if (m->elev[c] <= (m->bedrock[c] + active)) wet_factor = 10 * m->DX;
        for (int k = 0; k < 8; k++) {
          unsigned x2 = x + ox[k], y2 = y + oy[k];
          const bool diag = (ox[k] != 0 && oy[k] != 0);
          double drop = diag ? ((m->elev[c] - m->E(x2, y2)) / 1.41) : (m->elev[c] - m->E(x2, y2));
          if (drop > wet_factor && m->E(x2, y2) > -9999) {
            double diff = diag ? (((m->elev[c] - m->E(x2, y2)) / 1.41) - wet_factor)
                               : ((m->elev[c] - m->E(x2, y2)) - wet_factor);
            if ((m->elev[c] - diff) < (m->bedrock[c] + active))
              diff = (m->elev[c] - (m->bedrock[c] + active));
            if (diff > EF) diff = EF;
            m->elev[c] -= diff;
            m->E(x2, y2) += diff;
            total += diff;
          }
        }
      }
  } while (total > 0 && inc < 200);
}

// ---------------------------------------------------------------------------
// set-up and the main loop (main.cpp:102-204)
// ---------------------------------------------------------------------------
extern "C" void hco_prepare(hco_model* m) {
  for (unsigned i = 1; i < m->imax; i++)  // count_catchment_gridcells :2813
    for (unsigned j = 1; j < m->jmax; j++)
      if (m->E(i, j) > -9999) m->nActualGridCells[m->rfarea[m->ix(i, j)]]++;
  m->creep_time = m->creep_time2 = m->time_1 = m->cycle;  // set_time_counters :1862
  if (m->p.spatially_complex_rainfall) {
    topmodel_runoff_grid(m, 1.0);  // initialise_rainfall_runoff :2041-2053
    return;                        // initialise_drainage_area skips both :2055-2070
  }
  topmodel_runoff(m, 1.0);                                 // initialise_rainfall_runoff
  zero_and_calc_drainage_area(m);                          // initialise_drainage_area
  get_catchment_input_points(m);
}

extern "C" long hco_iterate(hco_model* m, long n, int flags, hco_step_record* rec) {
  long it = 0;
  const hc_params& p = m->p;
  // the main loop has ended (:1838): nothing runs, as in hc_run
  if (m->counter > 0 && !(m->cycle / 60 < p.maxcycle)) return 0;
  do {
    m->previous = m->cycle;                       // set_loop_cycle
    m->iod = std::abs(m->waterinput - m->waterOut);  // set_inputoutput_diff
    hco_set_maximum_timestep(m);
    m->counter++;                                 // increment_counters
    m->cycle += m->time_step / 60;
    reach_water_and_sediment_input(m);
    m->waterinput = 0;                            // catchment_waterinputs :2027
    if (p.spatially_complex_rainfall)
      catchment_water_input_grid(m, hco_get_flow_timestep(m));
    else
      catchment_water_input_and_hydrology(m, hco_get_flow_timestep(m));
    hco_flow_route(m);
    hco_depth_update(m);
    const double md = m->maxdepth;
    if ((m->counter % p.scan_area_interval_iter) == 0) hco_scan_area(m);
    if (!p.hydro_only) {
      if (m->counter >= m->erode_call) {          // call_erosion :2277
        m->erode_mult = x86_trunc_to_int(p.ERODEFACTOR / hco_erode(m, m->erode_mult));
        if (m->erode_mult < 1) m->erode_mult = 1;
        if (m->erode_mult > 5) m->erode_mult = 5;
        m->erode_call = m->counter + m->erode_mult;
      }
      if ((flags & HC_RUN_LATERAL) && m->counter >= m->lateralcounter) {  // call_lateral
        hco_lateral_channel_erode(m);
        m->lateralcounter = m->counter + (50 * m->erode_mult);
      }
    }
    hco_water_flux_out(m);
    if (!p.hydro_only && (m->counter % p.in_channel_landslide_iter_interval) == 0)
      hco_in_channel_landsliding(m);
    if (!(flags & HC_RUN_NOHILL)) {
      if (!p.hydro_only && (m->cycle > m->creep_time)) {
        m->creep_time += p.creep_time_interval;
        hco_creep(m, p.creep_coeff);
      }
      if (!p.hydro_only && m->cycle > m->creep_time2) {
        m->creep_time2 += p.global_landsliding_interval;
        hco_global_landsliding(m);
      }
    }
    if (rec) {
      hco_step_record& r = rec[it];
      r.counter = m->counter;
      r.cycle = m->cycle;
      r.time_step = m->time_step;
      r.maxdepth = md;
      r.waterOut = m->waterOut;
      r.waterinput = m->waterinput;
      r.erode_mult = m->erode_mult;
      r.sediQ = m->sediQ;
      r.globalsediq = m->globalsediq;
      r.baseflow = m->baseflow;
      const double a2 = m->DX * m->DX;
      r.vol_in = m->vin_it * a2;
      r.vol_out = (m->vout_it + m->vlost_it) * a2;
      r.vol_mask = m->vmask_it * a2;
      r.volume = (m->vol_scan_counter == m->counter) ? m->vol_scan * a2 : std::nan("");
    }
    m->vin_it = m->vout_it = m->vlost_it = m->vmask_it = 0;
    it++;
    if (m->grain_full) break;
    if (n >= 0 && it >= n) break;
  } while (m->cycle / 60 < p.maxcycle);
  return it;
}

// ---------------------------------------------------------------------------
// field / scalar access
// ---------------------------------------------------------------------------
namespace {
struct FieldRef {
  void* ptr;
  int64_t n;
  int elsize;
};
FieldRef lookup(hco_model* m, const char* name) {
  std::string s(name);
#define F(nm, vec) \
  if (s == nm) return FieldRef{(void*)m->vec.data(), (int64_t)m->vec.size(), (int)sizeof(m->vec[0])};
  F("elev", elev) F("water_depth", water_depth) F("qx", qx) F("qy", qy) F("qxs", qxs)
  F("qys", qys) F("Vsusptot", Vsusptot) F("Vel", Vel) F("Tau", Tau) F("bedrock", bedrock)
  F("spat_var_mannings", spat_var_mannings) F("area", area) F("ss", ss) F("vel_dir", vel_dir)
  F("sr", sr) F("sl", sl) F("su", su) F("sd", sd) F("grain", grain) F("strata", strata)
  F("index", index) F("down_scan", down_scan) F("rfarea", rfarea)
  F("inputpointsarray", inputpointsarray) F("edge", edge) F("edge2", edge2) F("veg", veg)
  F("cin_x", cin_x) F("cin_y", cin_y)
#undef F
  return FieldRef{nullptr, -1, 0};
}
}  // namespace

extern "C" int64_t hco_field_size(hco_model* m, const char* name) { return lookup(m, name).n; }
extern "C" int hco_field_elsize(hco_model* m, const char* name) { return lookup(m, name).elsize; }
extern "C" void* hco_field(hco_model* m, const char* name) { return lookup(m, name).ptr; }

extern "C" double hco_get_scalar(hco_model* m, const char* name) {
  std::string s(name);
#define S(nm, expr) \
  if (s == nm) return (double)(expr);
  S("cycle", m->cycle) S("time_step", m->time_step) S("maxdepth", m->maxdepth)
  S("waterinput", m->waterinput) S("waterOut", m->waterOut) S("counter", m->counter)
  S("erode_call", m->erode_call) S("erode_mult", m->erode_mult)
  S("lateralcounter", m->lateralcounter) S("time_1", m->time_1) S("baseflow", m->baseflow)
  S("grain_array_tot", m->grain_array_tot) S("grain_full", m->grain_full ? 1.0 : 0.0)
  S("sediQ", m->sediQ)
  S("globalsediq", m->globalsediq) S("tempbmax", m->tempbmax)
  S("totalinputpoints", m->totalinputpoints) S("temptot", m->temptot)
  S("mannings", m->mannings) S("j_mean1", m->j_mean.size() > 1 ? m->j_mean[1] : 0)
  S("nActualGridCells1", m->nActualGridCells.size() > 1 ? m->nActualGridCells[1] : 0)
#undef S
  if (s.rfind("sum_grain", 0) == 0) return m->sum_grain[std::atoi(s.c_str() + 9)];
  return NAN;
}

extern "C" int hco_set_scalar(hco_model* m, const char* name, double v) {
  std::string s(name);
  if (s == "cycle") m->cycle = v;
  else if (s == "previous") m->previous = v;
  else if (s == "time_step") m->time_step = v;
  else if (s == "maxdepth") m->maxdepth = v;
  else if (s == "waterinput") m->waterinput = v;
  else if (s == "waterOut") m->waterOut = v;
  else if (s == "counter") m->counter = (int)v;
  else if (s == "erode_call") m->erode_call = v;
  else if (s == "erode_mult") m->erode_mult = v;
  else if (s == "lateralcounter") m->lateralcounter = v;
  else if (s == "time_1") m->time_1 = v;
  else if (s == "baseflow") m->baseflow = v;
  else if (s == "grain_array_tot") m->grain_array_tot = (int)v;
  else if (s == "sediQ") m->sediQ = v;
  else if (s == "globalsediq") m->globalsediq = v;
  else if (s == "creep_time") m->creep_time = v;
  else if (s == "creep_time2") m->creep_time2 = v;
  else if (s.rfind("j_mean", 0) == 0) m->j_mean[std::atoi(s.c_str() + 6)] = v;
  else if (s.rfind("sum_grain", 0) == 0) m->sum_grain[std::atoi(s.c_str() + 9)] = v;
  else return -1;
  return 0;
}

// Continues from a state loaded field by field (e.g. a GPU snapshot): the
// catchment cell counts from the elevations, the TOPMODEL recurrence replayed
// to time_1 (it depends only on the rain table), the input points from the
// drainage area at the current baseflow.  Scalars must be set first.
extern "C" void hco_resume(hco_model* m) {
  for (size_t k = 0; k < m->nActualGridCells.size(); k++) m->nActualGridCells[k] = 0;
  for (unsigned i = 1; i < m->imax; i++)
    for (unsigned j = 1; j < m->jmax; j++)
      if (m->E(i, j) > -9999) m->nActualGridCells[m->rfarea[m->ix(i, j)]]++;
  const int rf = m->p.rfnum;
  if (m->p.spatially_complex_rainfall) {
    // the runoff grid from its start: every cell's recurrence depends only
    // on the rain table and its own elevation's no-data test
    std::fill(m->rj.begin(), m->rj.end(), 0.000000001);
    std::fill(m->rjo.begin(), m->rjo.end(), 0.000000001);
    std::fill(m->rold.begin(), m->rold.end(), 0.0);
    std::fill(m->rnew.begin(), m->rnew.end(), 0.0);
    topmodel_runoff_grid(m, 1.0);
    for (int t = 1; t <= (int)m->time_1; t++) topmodel_runoff_grid(m, (double)t);
    calchydrograph_grid(m, m->time_1 - m->cycle);
    return;
  }
  std::vector<double> keep(m->j_mean);
  for (int n = 0; n <= rf; n++) {
    m->jv[n] = m->jo[n] = 0.000000001;
    m->old_j_mean[n] = m->new_j_mean[n] = 0;
  }
  topmodel_runoff(m, 1.0);
  for (int t = 1; t <= (int)m->time_1; t++) topmodel_runoff(m, (double)t);
  m->j_mean = keep;
  zero_and_calc_drainage_area(m);
  get_catchment_input_points(m);
}
