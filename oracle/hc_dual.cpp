// Forward-mode (dual-number) derivative of the hydro-only iteration - test
// infrastructure for the device adjoint (hc_adjoint.cu), which has no
// counterpart in the reference.
//
// A plain FP64 restatement of one hydro-only iteration of the reference
// with every value carried as a dual number x + x'e (e^2 = 0):
//   catchment input points  catchment_water_input_and_hydrology :3463-3477
//   flow_route              :3063-3247 (hydro-only: no qxs/qys/vel_dir)
//   depth_update            :3259-3299
//   scan_area               :3821-3849 (every scan_area_interval_iter)
//   water_flux_out          :3005-3047
// The time steps and TOPMODEL j come from the device run being checked
// (the adjoint holds them fixed too); the input points are listed from the
// drainage area as get_catchment_input_points (:3741-3767) does, again
// whenever the baseflow threshold moves (:3524-3539).  The derivative seeds
// are a direction in Manning's n (dman) and one in the elevations (delev;
// either may be null); the branch tests use the values, as the adjoint's
// recorded run does.  Returns the number of outlet-Q samples, the loss over
// them and its directional derivative.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct D {
  double v, d;
};
inline D mk(double v) { return {v, 0.0}; }
inline D operator+(D a, D b) { return {a.v + b.v, a.d + b.d}; }
inline D operator-(D a, D b) { return {a.v - b.v, a.d - b.d}; }
inline D operator*(D a, D b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline D operator/(D a, D b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline D dsqrt(D a) {
  const double s = std::sqrt(a.v);
  return {s, a.d / (2 * s)};
}
inline D dabs(D a) { return a.v < 0 ? D{-a.v, -a.d} : a; }
inline D dmax(D a, D b) { return (a.v < b.v) ? b : a; }  // std::max

}  // namespace

extern "C" int hco_dual_run(
    int imax, int jmax, double DX, const double* elev, const double* man, const double* dman,
    const double* delev, const int32_t* rfarea, double* h_io, double* qx_io, double* qy_io, uint8_t* mask_io,
    const double* area, double baseflow, double min_q, double min_q_max, int rfnum,
    const double* nact,                            // per zone (0..16)
    int64_t n, const double* rec, int rec_stride,  // per iteration: [1] input dt, [2] flow dt, [3+z] j
    const double* time_step, const double* cycle, double cycle0, double counter0,
    int scan_interval, double hflow_threshold, double froude_limit, double edgeslope,
    double erodefactor, double threshold, const double* target, int64_t n_target,
    double* loss, double* dloss) {
  const size_t W = (size_t)jmax + 2, N2 = (size_t)(imax + 2) * W;
  const double g = 9.81;
  std::vector<D> h(N2), qx(N2), qy(N2), nn(N2), E(N2);
  for (size_t k = 0; k < N2; k++) {
    E[k] = D{elev[k], delev ? delev[k] : 0.0};
    h[k] = mk(h_io[k]);
    qx[k] = mk(qx_io[k]);
    qy[k] = mk(qy_io[k]);
    nn[k] = D{man[k], dman ? dman[k] : 0.0} * D{man[k], dman ? dman[k] : 0.0};
  }
  std::vector<uint8_t> mask(mask_io, mask_io + N2);
  std::vector<D> Q;
  std::vector<int32_t> cin_x(1), cin_y(1);
  double counters[17] = {0};
  int total_points = 0;
  auto points = [&]() {
    int t = 0;
    for (int z = 1; z <= rfnum; z++) counters[z] = 0;
    cin_x.assign(1, 0);
    cin_y.assign(1, 0);
    for (int i = 1; i <= imax; i++)
      for (int j = 1; j <= jmax; j++) {
        const double q = area[(size_t)i * W + j] * baseflow * 3 * DX * DX;
        if (q > min_q && q < min_q_max) {
          t++;
          cin_x.push_back(i);
          cin_y.push_back(j);
          counters[rfarea[(size_t)i * W + j]] += 1;
        }
      }
    total_points = t;  // the tests keep t > 0
  };
  points();
  double prev = cycle0, counter = counter0;
  auto face = [&](D q, D e0, D h0, D e1, D h1, D n2, double dt, int es) -> D {
    const D a0 = e0 + h0, a1 = e1 + h1;
    const D hflow = dmax(a0, a1) - dmax(e1, e0);
    if (!(hflow.v > hflow_threshold)) return mk(0.0);
    D slope = (a1 - a0) / mk(DX);
    if (es == 1) slope = mk(edgeslope);
    if (es == -1) slope = mk(0 - edgeslope);
    const D ghd = mk(g) * hflow * mk(dt);
    const D h3 = hflow * hflow * hflow;
    D qn = (q - ghd * slope) / (mk(1.0) + ghd * n2 * dabs(q) / h3);
    if (qn.v > 0 && ((qn / hflow) / dsqrt(mk(g) * hflow)).v > froude_limit)
      qn = hflow * (dsqrt(mk(g) * hflow) * mk(froude_limit));
    if (qn.v < 0 && (dabs(qn / hflow) / dsqrt(mk(g) * hflow)).v > froude_limit)
      qn = mk(0.0) - (hflow * (dsqrt(mk(g) * hflow) * mk(froude_limit)));
    if (qn.v > 0 && (qn * mk(dt) / mk(DX)).v > (h0 / mk(4.0)).v) qn = ((h0 * mk(DX)) / mk(5.0)) / mk(dt);
    if (qn.v < 0 && dabs(qn * mk(dt) / mk(DX)).v > (h1 / mk(4.0)).v)
      qn = mk(0.0) - ((h1 * mk(DX)) / mk(5.0)) / mk(dt);
    return qn;
  };
  for (int64_t t = 0; t < n; t++) {
    const double* r = rec + (size_t)t * rec_stride;
    const double idt = r[1], fdt = r[2], ts = time_step[t];
    counter += 1;
    // input points
    for (int z = 1; z <= total_points; z++) {
      const size_t cell = (size_t)cin_x[z] * W + cin_y[z];
      const int rf = rfarea[cell];
      double amt = (r[3 + rf] * nact[rf]) / (counters[rf]) * idt;
      if (amt > erodefactor) amt = erodefactor;
      h[cell] = h[cell] + mk(amt);
    }
    // flow_route over the mask, in any order (faces are independent)
    std::vector<D> nqx(qx), nqy(qy);
    for (int i = 1; i <= imax; i++)
      for (int j = 1; j <= jmax; j++) {
        const size_t cell = (size_t)i * W + j;
        if (!mask[cell] || !(elev[cell] > -9999)) continue;
        const D n2 = nn[cell];
        if ((h[cell].v > 0 || h[cell - W].v > 0) && elev[cell - W] > -9999)
          nqx[cell] = face(qx[cell], E[cell], h[cell], E[cell - W], h[cell - W], n2, fdt,
                           (i == imax) ? 1 : ((i <= 2) ? -1 : 0));
        if ((h[cell].v > 0 || h[cell - 1].v > 0) && elev[cell - 1] > -9999)
          nqy[cell] = face(qy[cell], E[cell], h[cell], E[cell - 1], h[cell - 1], n2, fdt,
                           (j == jmax) ? 1 : ((j <= 2) ? -1 : 0));
      }
    qx.swap(nqx);
    qy.swap(nqy);
    // depth_update
    for (int i = 1; i <= imax; i++)
      for (int j = 1; j <= jmax; j++) {
        const size_t cell = (size_t)i * W + j;
        if (!mask[cell]) continue;
        h[cell] = h[cell] + mk(fdt) * (qx[cell + W] - qx[cell] + qy[cell + 1] - qy[cell]) / mk(DX);
        if (h[cell].v > 0 && elev[cell] == -9999) h[cell] = mk(0.0);
      }
    // scan_area
    if (((long long)counter % scan_interval) == 0) {
      for (int i = 1; i <= imax; i++)
        for (int j = 1; j <= jmax; j++) {
          const size_t cell = (size_t)i * W + j;
          bool wet = false;
          for (int dx = -1; dx <= 1; dx++)
            for (int dy = -1; dy <= 1; dy++) wet |= h[cell + dx * (long)W + dy].v > 0;
          mask[cell] = wet ? 1 : 0;
        }
    }
    // water_flux_out
    D tot = mk(0.0);
    auto out = [&](int i, int j) {
      D& hh = h[(size_t)i * W + j];
      if (hh.v > threshold) {
        tot = tot + (hh - mk(threshold)) * mk(DX * DX / ts);
        hh = mk(threshold);
      }
    };
    for (int i = 1; i <= imax; i++) {
      out(i, jmax);
      out(i, 1);
    }
    for (int j = 1; j <= jmax; j++) {
      out(1, j);
      out(imax, j);
    }
    if (std::floor(cycle[t]) > std::floor(prev)) Q.push_back(tot);
    prev = cycle[t];
    // the baseflow tests of this iteration, with the j it computed (the j
    // the next iteration's inputs use)
    if (t + 1 < n) {
      const double* rn = rec + (size_t)(t + 1) * rec_stride;
      double jmeanmax = 0;
      for (int z = 1; z <= rfnum; z++)
        if (rn[3 + z] > jmeanmax) jmeanmax = rn[3 + z];
      bool recalc = false;
      if (jmeanmax >= baseflow) {
        baseflow = baseflow * 3;
        recalc = true;
      }
      if (baseflow > (jmeanmax * 3) && baseflow > 0.000001) {
        baseflow = jmeanmax * 1.25;
        recalc = true;
      }
      if (recalc) points();
    }
  }
  const int64_t S = std::min<int64_t>((int64_t)Q.size(), n_target);
  D L = mk(0.0);
  for (int64_t k = 0; k < S; k++) {
    const D e = Q[(size_t)k] - mk(target[k]);
    L = L + e * e / mk((double)S);
  }
  *loss = L.v;
  *dloss = L.d;
  for (size_t k = 0; k < N2; k++) {
    h_io[k] = h[k].v;
    qx_io[k] = qx[k].v;
    qy_io[k] = qy[k].v;
  }
  std::memcpy(mask_io, mask.data(), N2);
  return (int)Q.size();
}
