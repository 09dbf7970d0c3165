// Adjoint of the hydraulic iteration (no counterpart in the reference).
//
// For hydro-only catchment runs: the loss is the mean squared difference
// between the outlet discharge (water_flux_out's sum, :3005-3047) at the
// first iteration of every simulated minute and a target series.  Its
// gradient with respect to every cell's Manning's n and to every entry of
// the rain table is obtained by reverse-mode differentiation of the
// iteration as the device runs it:
//   catchment input points  h += min(j*N/count*dt, ERODEFACTOR)   (:3463-3477)
//   flow_route              the inertial face update and its limiters
//                           (:3063-3247), differentiated branch by branch
//   depth_update            h += dt*(div q)/DX                     (:3259-3299)
//   water_flux_out          edge clamp to the threshold, Q = sum
// with the time steps, the wet mask and the input points held at their
// recorded values (they are piecewise constant in the parameters).  The
// rain enters through TOPMODEL's j (host_topmodel_tangent).
//
// Memory: the state (h, qx, qy and the small run state) is checkpointed at
// segment starts (every K iterations, binomial schedule) during the forward
// run; the reverse pass replays one segment at a time from its checkpoint,
// keeping every iteration's state of the segment, and runs the adjoint
// iterations backwards through it.  With two slot sets, the replay of a
// segment (the model's stream) overlaps the adjoint iterations of the
// segment after it (a second stream).

#include "hc_internal.cuh"

#include <chrono>
#include <functional>
#include <memory>
#include <cmath>
#include <cstring>
#include <vector>

#define HC_TRY(expr)                         \
  do {                                       \
    hc_status st_ = (expr);                  \
    if (st_ != HC_OK) return st_;            \
  } while (0)
#define HC_CU(expr, what) HC_TRY(hc_cuda(c, (expr), what))

namespace {

constexpr double kG = 9.81;

// value and partial derivatives of a face discharge with respect to the
// previous discharge q, the two depths, n^2 and the two elevations
struct DQ {
  double v, dq, dh0, dh1, dnn, de0, de1;
};

// Three-way test of A > B from float estimates (as the forward kernel's):
// +1 surely, -1 surely not, 0 too close to call.
__device__ __forceinline__ int decide(float a, float b) {
  const float m = 1e-4f * (fabsf(a) + fabsf(b));
  if (!(m >= 1e-34f) || !(m < 1e30f)) return 0;
  const float dd = a - b;
  if (dd > m) return 1;
  if (dd < -m) return -1;
  return 0;
}

// The depth limits' exact tests (:3138, :3144), out of line: the float
// estimate decides almost every face, and inlined, these FP64 instructions
// would take FP64 issue slots at every call site whether they run or not.
static __device__ __noinline__ bool adj_depth_exceeds(double qn, double dt, double DX, double h) {
  return (qn * dt / DX) > (h / 4);
}
static __device__ __noinline__ bool adj_depth_exceeds_neg(double qn, double dt, double DX,
                                                          double h) {
  return fabs(qn * dt / DX) > (h / 4);
}
// The other rare paths, out of line too (smaller code: fewer instruction
// fetch stalls): the limits' value (x * DX / 5) / dt, the Froude test's exact
// form and sqrt(g hflow).
static __device__ __noinline__ double adj_limit_value(double x, double DX, double dt) {
  return ddiv_rn(ddiv_rn(x * DX, 5.0), dt);
}
static __device__ __noinline__ bool adj_froude_exceeds(double qn, double hflow, double fl) {
  return dgt(ddiv_rn(fabs(ddiv_rn(qn, hflow)), isqrt_rn(kG * hflow)), fl);
}
static __device__ __noinline__ double adj_sqrt_ghf(double hflow) { return isqrt_rn(kG * hflow); }
// the face's divisions through one out-of-line copy: inlined at each of its
// call sites, the integer-pipe division made the code large enough that
// instruction fetch stalled the warps (as in the forward kernel)
static __device__ __noinline__ double adj_div(double a, double b) { return ddiv_rn(a, b); }

// One face (:3096-3191), as the device evaluates it, with derivatives.
// The value and the branch decisions are the forward kernel's (exact FP64
// where a branch is decided, float estimates first, as there); the
// derivatives, which need no exact rounding, use reciprocals.  hflow =
// max(surfaces) - max(beds) and dA = a1 - a0 come from the caller (which
// decided hflow > hflow_threshold), with e0max = (e1 < e0); a1 > a0 exactly
// when dA > 0.  h0 and h1 are read only by the depth limits.  Comparisons
// run on the integer pipe (dkey etc.), as in the forward kernel.
template <class H0, class H1>
__device__ DQ face_dq(double q, double hflow, double dA, bool e0max, H0 h0f, H1 h1f, double nn,
                      double dt, int es, const hc_params& p, double rDX, const hc_divisor& dxd,
                      float DXf, float flf) {
  const double DX = p.DX;
  DQ r = {0, 0, 0, 0, 0, 0, 0};
  const bool a1max = dgt0(dA);
  // hflow = max(surfaces) - max(beds): its derivatives by the depths, and
  // by the elevations (through both maxima)
  const double dhf0 = a1max ? 0.0 : 1.0, dhf1 = a1max ? 1.0 : 0.0;
  const double dhfe0 = dhf0 - (e0max ? 1.0 : 0.0), dhfe1 = dhf1 - (e0max ? 0.0 : 1.0);
  double slope = ddiv_by(dA, dxd), ds0 = -rDX, ds1 = rDX;
  if (es == 1) slope = p.edgeslope, ds0 = ds1 = 0;
  if (es == -1) slope = zero_minus(p.edgeslope), ds0 = ds1 = 0;
  const double ghd = kG * hflow * dt;
  const double rhf = adj_div(1.0, hflow);
  // qn and its derivatives with respect to q, hflow, slope, nn
  double qn, d_q, d_hf, d_s, d_nn;
  if (deq0(q)) {
    qn = q - (ghd * slope);
    d_q = 1;
    d_hf = -kG * dt * slope;
    d_s = -ghd;
    d_nn = 0;
  } else {
    const double aq = __longlong_as_double(dbits(q) & 0x7fffffffffffffffLL);  // fabs
    const double c3 = icube_rn(hflow);
    const double F = adj_div(ghd * nn * aq, c3);
    const double D = 1 + F, N = q - (ghd * slope);
    qn = adj_div(N, D);
    const double rD = adj_div(1.0, D), rc3 = adj_div(1.0, c3);
    const double dF_q = ghd * nn * (dgt0(q) ? 1.0 : -1.0) * rc3;
    const double dF_hf = -2 * F * rhf;
    const double dF_nn = ghd * aq * rc3;
    d_q = rD - qn * dF_q * rD;
    d_hf = (-kG * dt * slope) * rD - qn * dF_hf * rD;
    d_s = -ghd * rD;
    d_nn = -qn * dF_nn * rD;
  }
  double dh0 = d_hf * dhf0 + d_s * ds0, dh1 = d_hf * dhf1 + d_s * ds1;
  // the slope reads the surfaces e + h, so an elevation moves it like a depth
  double de0 = d_hf * dhfe0 + d_s * ds0, de1 = d_hf * dhfe1 + d_s * ds1;
  // Froude limit (:3124-3134): |q/hflow| / sqrt(g*hflow) > froude_limit
  const double fl = p.froude_limit;
  if (!deq0(qn)) {
    const float hf = approx_abs_f(hflow);
    int t = decide(approx_abs_f(qn) / (hf * sqrtf(9.81f * hf)), flf);
    if (t == 0) t = adj_froude_exceeds(qn, hflow, fl) ? 1 : -1;
    if (t > 0) {
      const double sg = adj_sqrt_ghf(hflow);
      const double g = 1.5 * sg * fl;
      if (dgt0(qn)) {
        qn = hflow * (sg * fl);
        d_q = 0, d_nn = 0, dh0 = g * dhf0, dh1 = g * dhf1, de0 = g * dhfe0, de1 = g * dhfe1;
      } else {
        qn = zero_minus(hflow * (sg * fl));
        d_q = 0, d_nn = 0, dh0 = -g * dhf0, dh1 = -g * dhf1, de0 = -g * dhfe0, de1 = -g * dhfe1;
      }
    }
  }
  // depth limits (:3138-3148), one after the other
  const float dtf = approx_abs_f(dt);
  if (dgt0(qn)) {
    const double h0 = h0f();
    int t = decide(approx_abs_f(qn) * dtf / DXf, approx_f(h0) * 0.25f);
    if (t == 0) t = adj_depth_exceeds(qn, dt, DX, h0) ? 1 : -1;
    if (t > 0) {
      qn = adj_limit_value(h0, DX, dt);
      d_q = 0, d_nn = 0, dh0 = adj_limit_value(1.0, DX, dt), dh1 = 0, de0 = de1 = 0;
    }
  }
  if (dlt0(qn)) {
    const double h1 = h1f();
    int t = decide(approx_abs_f(qn) * dtf / DXf, approx_f(h1) * 0.25f);
    if (t == 0) t = adj_depth_exceeds_neg(qn, dt, DX, h1) ? 1 : -1;
    if (t > 0) {
      qn = zero_minus(adj_limit_value(h1, DX, dt));
      d_q = 0, d_nn = 0, dh0 = 0, dh1 = -adj_limit_value(1.0, DX, dt), de0 = de1 = 0;
    }
  }
  r.v = qn;
  r.dq = d_q;
  r.dh0 = dh0;
  r.dh1 = dh1;
  r.dnn = d_nn;
  r.de0 = de0;
  r.de1 = de1;
  return r;
}

struct AdjStep {
  double fdt, ts, input_dt, gQ;  // flow dt, time_step at water_flux_out, dL/dQ
  double amt[HC_MAX_RF + 1];     // input amount per zone
  double damt[HC_MAX_RF + 1];    // d amount / d j per zone (0 where clamped)
};

struct AdjBufs {
  // one iteration of the segment: state before it
  const double *h0, *qx0, *qy0;
  const uint8_t* mask;
  // discharges after it
  const double *qx1, *qy1;
  const uint8_t* point;  // input-point cells of this iteration
  double *lam, *mux, *muy;  // adjoints of h, qx, qy (in: after, out: before)
  double *lamd, *p0x, *p0y, *p1x, *p1y;
  // elevation terms: the x and y faces' own-cell terms, to the cell above,
  // to the left; the faces' n terms (dL/d(n^2) by face)
  double *pe0x, *pe0y, *pe1x, *pe1y, *gx, *gy;
  double *gn;   // accumulated dL/dn per cell
  double *ge;   // accumulated dL/d(elevation) per cell
  uint8_t *pflag;  // the cell's face terms (p*, pe*) may be nonzero
  double *gj;   // dL/dj per zone for this iteration
};

__device__ __forceinline__ bool edge_cell(const hc_view& c, int i, int j) {
  return i == 1 || i == c.imax || j == 1 || j == c.jmax;
}

// A cell outside the wet list that is no input point and no edge cell
// keeps its depth through an iteration: its depth adjoint passes through
// unchanged (k_adj_depth leaves lamd unwritten there; readers take lam),
// and a cell whose faces and whose up and left neighbours are all outside
// the list has no face terms (its p* entries are zero; pflag says which
// entries may not be).  Dry parts of the grid so cost a few bytes a cell.
__device__ __forceinline__ bool depth_active(const hc_view& c, const AdjBufs& b, size_t cell,
                                             int i, int j) {
  return b.mask[cell] || b.point[cell] || i == 1 || i == c.imax || j == 1 || j == c.jmax;
}

// water_flux_out and depth_update, reversed: lamd = adjoint of the depth
// after inputs, through the depth update (0 for no-data cells it zeroes)
__global__ void k_adj_depth(const hc_view c, AdjBufs b, AdjStep st) {
  const int j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int i = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > c.imax || j > c.jmax) return;
  const size_t W = c.W, cell = (size_t)i * W + j;
  if (!depth_active(c, b, cell, i, j)) return;
  const int rf = c.rfarea[cell];
  double ha = b.h0[cell];
  if (b.point[cell] && rf >= 0 && rf <= HC_MAX_RF) ha += st.amt[rf];
  double hd = ha;
  bool zeroed = false;
  if (b.mask[cell]) {
    hd += ddiv_by(st.fdt * (b.qx1[cell + W] - b.qx1[cell] + b.qy1[cell + 1] - b.qy1[cell]),
                  c.dxd);
    if (dgt0(hd) && dbits(c.elev[cell]) == kNoDataBits) zeroed = true;
  }
  double lam = b.lam[cell];
  // water_flux_out clamps an edge cell above the threshold: its depth after
  // the iteration is a constant, and the excess went into Q
  if (edge_cell(c, i, j) && !zeroed && dgt(hd, c.p.water_depth_erosion_threshold))
    lam = st.gQ * c.p.DX * c.p.DX / st.ts;
  b.lamd[cell] = zeroed ? 0.0 : lam;
}

// flow_route reversed, face by face: discharge adjoints before the
// iteration, the depth terms each face passes to its two cells, the n and
// elevation terms.  Only the faces that flowed (hflow above the threshold)
// need face_dq, and in a storm about half the listed cells' faces do not:
// a warp running its 32 cells' faces in place would issue the FP64 work with
// a fraction of its lanes.  So each lane first forms its cell's discharge
// adjoints and writes out every face that needs no face_dq (a face of a cell
// that is not updated keeps its adjoint; one set to zero passes none); the
// faces that flowed are queued per warp with hflow, the surface difference
// and their discharge adjoint, and whenever 32 are queued the warp runs them
// together, the rest carried over to the warp's next 32 cells.  Each output
// entry is written once, by one lane.
constexpr int kAdjQ = 96;  // queue entries per warp: < 32 carried + 64 new

struct AdjQueue {
  uint32_t f[kAdjQ];  // cell << 2 | (e1 < e0) << 1 | y face
  double hf[kAdjQ], da[kAdjQ], mu[kAdjQ];
};

__device__ __forceinline__ double adj_hin(const hc_view& c, const AdjBufs& b, const AdjStep& st,
                                          size_t q) {
  double h = b.h0[q];
  if (b.point[q]) {
    const int rf = c.rfarea[q];
    if (rf >= 0 && rf <= HC_MAX_RF) h += st.amt[rf];
  }
  return h;
}

__device__ __forceinline__ void adj_face(const hc_view& c, const AdjBufs& b, const AdjStep& st,
                                         uint32_t f, double hflow, double dA, double mu) {
  const size_t W = c.W;
  const size_t cell = f >> 2;
  const bool yface = f & 1u, e0max = (f >> 1) & 1u;
  const size_t nb = yface ? cell - 1 : cell - W;
  const int i = (int)(cell / W), j = (int)(cell - (size_t)i * W);
  const hc_params& p = c.p;
  const double n = p.spatially_var_mannings ? c.man[cell] : p.mannings;
  const double nn = n * n;
  const int es = yface ? ((j == c.jmax) ? 1 : ((j <= 2) ? -1 : 0))
                       : ((i == c.imax) ? 1 : ((i <= 2) ? -1 : 0));
  const double q = yface ? b.qy0[cell] : b.qx0[cell];
  const DQ r = face_dq(
      q, hflow, dA, e0max, [&] { return adj_hin(c, b, st, cell); },
      [&] { return adj_hin(c, b, st, nb); }, nn, st.fdt, es, p, c.rDX, c.dxd, c.DXf, c.flf);
  if (yface) {
    b.muy[cell] = r.dq * mu;
    b.p0y[cell] = r.dh0 * mu;
    b.p1y[cell] = r.dh1 * mu;
    b.pe0y[cell] = r.de0 * mu;
    b.pe1y[cell] = r.de1 * mu;
    b.gy[cell] = r.dnn * mu;
  } else {
    b.mux[cell] = r.dq * mu;
    b.p0x[cell] = r.dh0 * mu;
    b.p1x[cell] = r.dh1 * mu;
    b.pe0x[cell] = r.de0 * mu;
    b.pe1x[cell] = r.de1 * mu;
    b.gx[cell] = r.dnn * mu;
  }
}

__device__ __forceinline__ void adj_zero_x(const AdjBufs& b, size_t cell) {
  b.p0x[cell] = b.p1x[cell] = b.pe0x[cell] = b.pe1x[cell] = b.gx[cell] = 0;
}
__device__ __forceinline__ void adj_zero_y(const AdjBufs& b, size_t cell) {
  b.p0y[cell] = b.p1y[cell] = b.pe0y[cell] = b.pe1y[cell] = b.gy[cell] = 0;
}

__global__ void __launch_bounds__(256, 4) k_adj_flow_c(const hc_view c, AdjBufs b, AdjStep st) {
  __shared__ AdjQueue qs[8];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  AdjQueue& Q = qs[warp];
  const size_t W = c.W;
  const int cpr = (c.jmax + 31) / 32;  // chunks of 32 columns per row
  const long long chunks = (long long)c.imax * cpr;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const double k = st.fdt / c.p.DX;
  int qn = 0;  // the same on every lane
  for (long long ch = (long long)blockIdx.x * (blockDim.x >> 5) + warp; ch < chunks; ch += warps) {
    const int i = 1 + (int)(ch / cpr);
    const int j = 1 + (int)(ch % cpr) * 32 + lane;
    bool fx = false, fy = false, ex = false, ey = false;
    size_t cell = 0;
    double mux = 0, muy = 0, hx = 0, ax = 0, hy = 0, ay = 0;
    if (j <= c.jmax) {
      cell = (size_t)i * W + j;
      if (!(b.mask[cell] || b.mask[cell - W] || b.mask[cell - 1])) {
        if (b.pflag[cell]) {
          adj_zero_x(b, cell);
          adj_zero_y(b, cell);
          b.pflag[cell] = 0;
        }
      } else {
        auto ml = [&](size_t q) { return b.mask[q] ? b.lamd[q] : 0.0; };
        mux = b.mux[cell] + k * (ml(cell - W) - ml(cell));
        muy = b.muy[cell] + k * (ml(cell - 1) - ml(cell));
        const double e0 = c.elev[cell];
        b.pflag[cell] = 1;
        if (!(b.mask[cell] && dkey(e0) > kNoDataKey)) {
          // flow_route leaves both faces alone
          b.mux[cell] = mux;
          b.muy[cell] = muy;
          adj_zero_x(b, cell);
          adj_zero_y(b, cell);
        } else {
          const double h0 = adj_hin(c, b, st, cell);
          const double a0 = e0 + h0;
          const bool wet0 = dgt0(h0);
          double ox = mux, oy = muy;
          {
            const size_t up = cell - W;
            const double h1 = adj_hin(c, b, st, up), e1 = c.elev[up];
            if ((wet0 || dgt0(h1)) && dkey(e1) > kNoDataKey) {
              const double a1 = e1 + h1;
              hx = imax_d(a0, a1) - imax_d(e1, e0);
              ax = a1 - a0;
              ex = dlt(e1, e0);
              fx = dkey(hx) > c.thr_key;
              if (!fx) ox = 0;  // q set to zero: no adjoint passes back
            }
          }
          {
            const size_t lf = cell - 1;
            const double h1 = adj_hin(c, b, st, lf), e1 = c.elev[lf];
            if ((wet0 || dgt0(h1)) && dkey(e1) > kNoDataKey) {
              const double a1 = e1 + h1;
              hy = imax_d(a0, a1) - imax_d(e1, e0);
              ay = a1 - a0;
              ey = dlt(e1, e0);
              fy = dkey(hy) > c.thr_key;
              if (!fy) oy = 0;
            }
          }
          if (!fx) {
            b.mux[cell] = ox;
            adj_zero_x(b, cell);
          }
          if (!fy) {
            b.muy[cell] = oy;
            adj_zero_y(b, cell);
          }
        }
      }
    }
    const unsigned bx = __ballot_sync(FULL, fx), by = __ballot_sync(FULL, fy);
    const unsigned below = (1u << lane) - 1u;
    const int nx = __popc(bx);
    if (fx) {
      const int s = qn + __popc(bx & below);
      Q.f[s] = ((uint32_t)cell << 2) | (ex ? 2u : 0u);
      Q.hf[s] = hx;
      Q.da[s] = ax;
      Q.mu[s] = mux;
    }
    if (fy) {
      const int s = qn + nx + __popc(by & below);
      Q.f[s] = ((uint32_t)cell << 2) | (ey ? 2u : 0u) | 1u;
      Q.hf[s] = hy;
      Q.da[s] = ay;
      Q.mu[s] = muy;
    }
    qn += nx + __popc(by);
    __syncwarp();
    while (qn >= 32) {
      qn -= 32;
      const uint32_t f = Q.f[qn + lane];
      const double hf = Q.hf[qn + lane], da = Q.da[qn + lane], mu = Q.mu[qn + lane];
      __syncwarp();  // the entries are read before the next cells' are written
      adj_face(c, b, st, f, hf, da, mu);
    }
  }
  if (lane < qn) adj_face(c, b, st, Q.f[lane], Q.hf[lane], Q.da[lane], Q.mu[lane]);
}

// the depth adjoint before the iteration (inputs add a constant), and the
// input points' dL/dj
__global__ void __launch_bounds__(256) k_adj_gather(const hc_view c, AdjBufs b, AdjStep st) {
  __shared__ double sj[8][HC_MAX_RF + 1];
  const int j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int i = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  const int warp = t >> 5, lane = t & 31;
  double mine = 0;
  int myrf = -1;
  const size_t W = c.W, cell = (size_t)i * W + j;
  const bool in = i <= c.imax && j <= c.jmax;
  const bool dact = in && depth_active(c, b, cell, i, j);
  if (in && (dact || b.pflag[cell] || b.pflag[cell + W] || b.pflag[cell + 1])) {
    const double la = (dact ? b.lamd[cell] : b.lam[cell]) + b.p0x[cell] + b.p0y[cell] +
                      b.p1x[cell + W] + b.p1y[cell + 1];
    b.lam[cell] = la;
    b.ge[cell] += (b.pe0x[cell] + b.pe0y[cell]) + b.pe1x[cell + W] + b.pe1y[cell + 1];
    if (b.pflag[cell]) {
      // the faces' n^2 terms, as dL/dn (n^2 = n*n)
      const double g2 = b.gx[cell] + b.gy[cell];
      if (!deq0(g2)) {
        const double n = c.p.spatially_var_mannings ? c.man[cell] : c.p.mannings;
        b.gn[cell] += g2 * 2 * n;
      }
    }
    const int rf = c.rfarea[cell];
    if (b.point[cell] && rf >= 0 && rf <= HC_MAX_RF) {
      mine = la * st.damt[rf];
      myrf = rf;
    }
  }
  // per zone: warp sums, then block sums, then one atomic per zone and block
  // (input points are few: a warp without one of the zone's sums to +0 with
  // no FP64 work)
  for (int z = 0; z <= c.p.rfnum && z <= HC_MAX_RF; z++) {
    double v = 0.0;
    if (__ballot_sync(0xffffffffu, myrf == z)) {
      v = (myrf == z) ? mine : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    if (lane == 0) sj[warp][z] = v;
  }
  __syncthreads();
  if (t <= c.p.rfnum && t <= HC_MAX_RF) {
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x * blockDim.y) / 32; w++) s += sj[w][t];
    if (s != 0) atomicAdd(&b.gj[t], s);
  }
}

// the state an adjoint replay keeps: before the iteration's inputs
__global__ void __launch_bounds__(256) k_adj_save(const hc_view c, const hc_dev* d) {
  if (!d->it_active) return;
  const int64_t k = d->adj_i - 1 - d->adj_slot_t0;  // k_control has counted this iteration
  if (k < 0 || k >= d->adj_slot_n) return;
  const size_t N2 = c.N2, off = (size_t)k * N2;
  double* __restrict__ sh = d->adj_slot_h + off;
  double* __restrict__ sqx = d->adj_slot_qx + off;
  double* __restrict__ sqy = d->adj_slot_qy + off;
  uint8_t* __restrict__ sm = d->adj_slot_mask + off;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < N2;
       q += (size_t)gridDim.x * blockDim.x) {
    sh[q] = c.h[q];
    sqx[q] = c.qx[q];
    sqy[q] = c.qy[q];
    sm[q] = c.mask[q];
  }
}

__global__ void k_point_flags(const hc_view c, uint8_t* flags, int total) {
  for (int z = 1 + blockIdx.x * blockDim.x + threadIdx.x; z <= total;
       z += gridDim.x * blockDim.x)
    flags[(size_t)c.cin_x[z] * c.W + c.cin_y[z]] = 1;
}

// ------------------------------------------------------------------ host
struct Dev {
  void* p = nullptr;
  ~Dev() { if (p) cudaFree(p); }
  template <class T> T* as() { return (T*)p; }
};

cudaError_t dmalloc(Dev& d, size_t bytes) { return cudaMalloc(&d.p, bytes ? bytes : 8); }

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// the run state a hydro-only iteration reads and writes
struct Checkpoint {
  Dev h, qx, qy, mask, border, wet, cinx, ciny, dev;
};

hc_status save_state(hc_ctx* c, Checkpoint& k, bool alloc) {
  hc_view& v = c->v;
  const size_t N2 = v.N2, nc = (size_t)v.cin_cap + 2;
  if (alloc) {
    if (dmalloc(k.h, N2 * 8) || dmalloc(k.qx, N2 * 8) || dmalloc(k.qy, N2 * 8) ||
        dmalloc(k.mask, N2) || dmalloc(k.border, N2) || dmalloc(k.wet, N2 * 4) ||
        dmalloc(k.cinx, nc * 4) ||
        dmalloc(k.ciny, nc * 4) || dmalloc(k.dev, sizeof(hc_dev)))
      return hc_fail(c, HC_ERR_NOMEM, "adjoint checkpoint: out of device memory");
  }
  cudaStream_t s = c->s;
  cudaMemcpyAsync(k.h.p, v.h, N2 * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(k.qx.p, v.qx, N2 * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(k.qy.p, v.qy, N2 * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(k.mask.p, v.mask, N2, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(k.border.p, v.border, N2, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(k.wet.p, v.wet, N2 * 4, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(k.cinx.p, v.cin_x, nc * 4, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(k.ciny.p, v.cin_y, nc * 4, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(k.dev.p, c->dev, sizeof(hc_dev), cudaMemcpyDeviceToDevice, s);
  return hc_cuda(c, cudaGetLastError(), "adjoint checkpoint");
}

hc_status load_state(hc_ctx* c, Checkpoint& k) {
  hc_view& v = c->v;
  const size_t N2 = v.N2, nc = (size_t)v.cin_cap + 2;
  cudaStream_t s = c->s;
  cudaMemcpyAsync(v.h, k.h.p, N2 * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(v.qx, k.qx.p, N2 * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(v.qy, k.qy.p, N2 * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(v.mask, k.mask.p, N2, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(v.border, k.border.p, N2, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(v.wet, k.wet.p, N2 * 4, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(v.cin_x, k.cinx.p, nc * 4, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(v.cin_y, k.ciny.p, nc * 4, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(c->dev, k.dev.p, sizeof(hc_dev), cudaMemcpyDeviceToDevice, s);
  if (cudaGetLastError() != cudaSuccess) return hc_fail(c, HC_ERR_CUDA, "adjoint restore");
  return ctx_pull(c);
}

// A segment's iteration states: h, qx, qy and the wet mask of K
// iterations (qx, qy one more: the discharges after the last), and the
// event that marks the last adjoint iteration that read them.
struct SlotSet {
  Dev h, qx, qy, mask;
  cudaEvent_t free_ev = nullptr;
  ~SlotSet() {
    if (free_ev) cudaEventDestroy(free_ev);
  }
};

// switches the time-step recording on (mode 1) or imposes recorded steps
// (mode 2) for the next iterations, from record index i0
// (k_adj_save keeps the states of iterations slot_t0 .. slot_t0+slot_n-1
// in the slot set `set`)
hc_status adj_mode(hc_ctx* c, double* buf, int64_t n, int mode, int64_t i0,
                   int64_t slot_t0 = 0, int64_t slot_n = 0, SlotSet* set = nullptr) {
  if (c->v.adj_dt != buf) {
    c->v.adj_dt = buf;
    c->graph_iters = 0;  // the graphs hold the view by value
  }
  HC_TRY(ctx_pull(c));
  c->hdev->adj_mode = buf ? mode : 0;
  c->hdev->adj_i = i0;
  c->hdev->adj_n = buf ? n : 0;
  c->hdev->adj_slot_t0 = slot_t0;
  c->hdev->adj_slot_n = set ? slot_n : 0;
  if (set) {
    c->hdev->adj_slot_h = set->h.as<double>();
    c->hdev->adj_slot_qx = set->qx.as<double>();
    c->hdev->adj_slot_qy = set->qy.as<double>();
    c->hdev->adj_slot_mask = set->mask.as<uint8_t>();
  }
  return ctx_push(c);
}

// input points of an adjoint replay: flag arrays, each valid from an
// iteration on (the points change only when the baseflow threshold moves)
struct PointsLog {
  std::vector<int64_t> start;
  std::vector<Dev*> flags;
  std::vector<std::vector<double>> nact, cnt;  // the counters the inputs divide by
  ~PointsLog() {
    for (Dev* f : flags) delete f;
  }
  hc_status add(hc_ctx* c, int64_t from) {
    Dev* f = new Dev();
    flags.push_back(f);
    start.push_back(from);
    const hc_scalars& sc = c->hdev->s;
    nact.emplace_back(sc.nActualGridCells, sc.nActualGridCells + HC_MAX_RF + 1);
    cnt.emplace_back(sc.catchment_input_counter, sc.catchment_input_counter + HC_MAX_RF + 1);
    // stream-ordered: no device-wide synchronisation while adjoint
    // iterations run on the other stream
    if (cudaMallocAsync(&f->p, c->v.N2, c->s) != cudaSuccess)
      return hc_fail(c, HC_ERR_NOMEM, "adjoint points");
    cudaMemsetAsync(f->p, 0, c->v.N2, c->s);
    k_point_flags<<<152 * 4, 256, 0, c->s>>>(c->v, f->as<uint8_t>(),
                                             (int)c->hdev->s.totalinputpoints);
    return hc_cuda(c, cudaGetLastError(), "adjoint points");
  }
  size_t version(int64_t t) const {
    size_t r = 0;
    for (size_t k = 0; k < start.size(); k++)
      if (start[k] <= t) r = k;
    return r;
  }
  const uint8_t* at(int64_t t) const { return flags[version(t)]->as<uint8_t>(); }
  const double* nact_at(int64_t t) const { return nact[version(t)].data(); }
  const double* cnt_at(int64_t t) const { return cnt[version(t)].data(); }
};

void points_hook(hc_ctx* c, void* arg) {
  ((PointsLog*)arg)->add(c, c->hdev->adj_i);
}

// sample rule: the first iteration whose cycle (minutes) passes a whole minute
void samples_of(const std::vector<hc_step_record>& rec, double cycle0, std::vector<int64_t>* at) {
  double prev = cycle0;
  for (size_t t = 0; t < rec.size(); t++) {
    if (std::floor(rec[t].cycle) > std::floor(prev)) at->push_back((int64_t)t);
    prev = rec[t].cycle;
  }
}

}  // namespace

extern "C" hc_status hc_adj_forward(hc_ctx* c, int64_t n, const double* fixed, double* rec_out,
                                    double* q_samples, int64_t q_cap, int64_t* n_samples) {
  if (!c || n <= 0) return HC_ERR_ARG;
  if (!c->v.p.hydro_only) return hc_fail(c, HC_ERR_UNSUPPORTED, "adjoint runs are hydro-only");
  if (c->v.p.spatially_complex_rainfall)
    return hc_fail(c, HC_ERR_UNSUPPORTED, "adjoint runs use the zoned rainfall inputs");
  if (!c->prepared) return hc_fail(c, HC_ERR_STATE, "hc_prepare must come before the run");
  Dev dt;
  const size_t nrec = (size_t)n * HC_ADJ_REC;
  HC_CU(dmalloc(dt, nrec * 8), "adjoint record");
  if (fixed) HC_CU(cudaMemcpy(dt.p, fixed, nrec * 8, cudaMemcpyHostToDevice), "adjoint record");
  HC_TRY(ctx_pull(c));
  const double cycle0 = c->hdev->s.cycle;
  HC_TRY(adj_mode(c, dt.as<double>(), n, fixed ? 2 : 1, 0));
  std::vector<hc_step_record> rec((size_t)n);
  int64_t done = 0;
  const hc_status st = hc_run(c, n, 0, rec.data(), &done);
  const hc_status st2 = adj_mode(c, nullptr, 0, 0, 0);
  if (st != HC_OK) return st;
  if (st2 != HC_OK) return st2;
  rec.resize((size_t)done);
  if (rec_out) HC_CU(cudaMemcpy(rec_out, dt.p, nrec * 8, cudaMemcpyDeviceToHost), "adjoint record");
  std::vector<int64_t> at;
  samples_of(rec, cycle0, &at);
  int64_t k = 0;
  for (int64_t t : at) {
    if (q_samples && k < q_cap) q_samples[k] = rec[(size_t)t].waterOut;
    k++;
  }
  if (n_samples) *n_samples = k;
  return HC_OK;
}

// ---- binomial checkpointing (Griewank's revolve, by recursion) -----------
// The run is cut into m segments of K iterations.  Reversing segments
// [a, b) with the state at a in a snapshot and s more snapshots free: one
// segment is a leaf (replay it from the state at a, keeping each
// iteration's state, then run its adjoint iterations last first); with no
// snapshot free, every segment from the last down is reached again from a;
// otherwise the state at a split point mid is made (advancing from a) and
// kept, [mid, b) is reversed with s-1 snapshots and [a, mid) with s.  With
// r the smallest repetition number with C(s+r, s) >= b-a, any mid with
// b-mid <= C(s-1+r, s-1) and mid-a <= C(s+r-1, s) gives the least
// recomputation (r advances per segment at most); this takes the first.
namespace {

double binom(int s, int r) {  // C(s + r, s), saturating
  double v = 1;
  for (int k = 1; k <= s; k++) {
    v = v * (r + k) / k;
    if (v > 1e18) return 1e18;
  }
  return v;
}

int repetitions(int64_t l, int s) {
  int r = 0;
  while (binom(s, r) < (double)l) r++;
  return r;
}

int64_t split_point(int64_t a, int64_t b, int s) {
  const int64_t l = b - a;
  const int r = repetitions(l, s);
  const double right = binom(s - 1, r);  // segments [mid, b) may hold
  int64_t m = (right >= (double)l) ? 1 : l - (int64_t)right;
  if (m < 1) m = 1;
  if (m > l - 1) m = l - 1;
  return a + m;
}

// segments advanced again to reverse [a, b) with s free snapshots (the
// leaves' replays not counted); on the right spine of the recursion the
// split points were kept by the forward run and cost nothing
double schedule_cost(int64_t a, int64_t b, int s, bool spine) {
  const int64_t l = b - a;
  if (l <= 1) return 0;
  if (s == 0) return (double)l * (l - 1) / 2;
  const int64_t mid = split_point(a, b, s);
  return (spine ? 0.0 : (double)(mid - a)) + schedule_cost(mid, b, s - 1, spine) +
         schedule_cost(a, mid, s, false);
}

struct Revolve {
  hc_ctx* c;
  int64_t n, K, m;            // iterations, segment length, segments
  std::vector<Checkpoint>* slots;
  std::vector<int64_t> slot_of;  // segment -> snapshot slot holding its start (-1 none)
  std::vector<int> free_slots;
  std::function<hc_status(int64_t)> leaf;          // reverse segment g from the state now
  std::function<hc_status(int64_t, int64_t)> advance;  // iterations [t0, t1) forward
  int64_t advances = 0;      // iterations advanced beyond the first sweep

  hc_status restore(int64_t g) { return load_state(c, (*slots)[(size_t)slot_of[(size_t)g]]); }
  hc_status keep(int64_t g) {
    if (free_slots.empty()) return hc_fail(c, HC_ERR_STATE, "adjoint: no snapshot slot left");
    const int k = free_slots.back();
    free_slots.pop_back();
    slot_of[(size_t)g] = k;
    return save_state(c, (*slots)[(size_t)k], false);
  }
  void drop(int64_t g) {
    if (slot_of[(size_t)g] >= 0 && g != 0) {
      free_slots.push_back((int)slot_of[(size_t)g]);
      slot_of[(size_t)g] = -1;
    }
  }
  hc_status reach(int64_t from, int64_t to) {  // segment boundaries
    HC_TRY(restore(from));
    if (to > from) {
      advances += std::min(n, to * K) - from * K;
      HC_TRY(advance(from * K, std::min(n, to * K)));
    }
    return HC_OK;
  }
  hc_status reverse(int64_t a, int64_t b, int s) {
    if (b - a == 1) {
      HC_TRY(restore(a));
      return leaf(a);
    }
    if (s == 0) {
      for (int64_t g = b - 1; g >= a; g--) {
        HC_TRY(reach(a, g));
        HC_TRY(leaf(g));
      }
      return HC_OK;
    }
    const int64_t mid = split_point(a, b, s);
    const bool had = slot_of[(size_t)mid] >= 0;  // kept by the first sweep
    if (!had) {
      HC_TRY(reach(a, mid));
      HC_TRY(keep(mid));
    }
    HC_TRY(reverse(mid, b, s - 1));
    drop(mid);
    return reverse(a, mid, s);
  }
};

}  // namespace

extern "C" hc_status hc_adj_gradient(hc_ctx* c, int64_t n, int32_t max_states,
                                     const double* q_target, int64_t n_target, double* loss,
                                     double* grad_n, double* grad_rain, double* grad_elev,
                                     double* ms) {
  if (!c || n <= 0 || max_states < 2 || !q_target || n_target < 0) return HC_ERR_ARG;
  hc_view& v = c->v;
  if (!v.p.hydro_only) return hc_fail(c, HC_ERR_UNSUPPORTED, "adjoint runs are hydro-only");
  if (v.p.spatially_complex_rainfall)
    return hc_fail(c, HC_ERR_UNSUPPORTED, "adjoint runs use the zoned rainfall inputs");
  if (!c->prepared) return hc_fail(c, HC_ERR_STATE, "hc_prepare must come before the run");
  if (v.N2 >= (size_t)1 << 30)  // k_adj_flow_c queues a face as cell << 2 | 2 bits
    return hc_fail(c, HC_ERR_UNSUPPORTED, "adjoint runs take grids of fewer than 2^30 cells");
  const auto t_all = std::chrono::steady_clock::now();
  const size_t N2 = v.N2;
  cudaStream_t s = c->s;
  // The states kept: snapshots (run state at a segment start) and the K
  // iteration states of a segment, max_states in all.  With two slot sets
  // the replay of one segment runs while the adjoint iterations of the one
  // after it read the other set (two streams); a second set costs K states.
  // Segment length and sets: the least recomputation; of those two sets,
  // then the longest segment (fewer, longer replays: less launch and host
  // overhead).
  int64_t K = 1;
  int snaps = 0, nsets = 1;
  {
    double best = 1e300;
    for (int sets = 1; sets <= 2; sets++)
      for (int64_t k = 1; sets * k < max_states && k <= n; k = (k < 8) ? k + 1 : k + k / 8) {
        const int sn = (int)(max_states - sets * k);  // snapshots, the initial state's included
        const int64_t m = (n + k - 1) / k;
        const double cost = schedule_cost(0, m, std::min<int64_t>(sn, m) - 1, true) * (double)k;
        if (cost < best || (cost == best && (sets > nsets || k > K))) {
          best = cost;
          K = k;
          snaps = sn;
          nsets = sets;
        }
      }
  }
  const int64_t nseg = (n + K - 1) / K;
  if (snaps > nseg) snaps = (int)nseg;
  if (nseg < 2) nsets = 1;
  SlotSet sets[2];
  for (int x = 0; x < nsets; x++) {
    SlotSet& S = sets[x];
    if (dmalloc(S.h, (size_t)K * N2 * 8) || dmalloc(S.qx, (size_t)(K + 1) * N2 * 8) ||
        dmalloc(S.qy, (size_t)(K + 1) * N2 * 8) || dmalloc(S.mask, (size_t)K * N2))
      return hc_fail(c, HC_ERR_NOMEM, "adjoint: out of device memory (segment of %lld)",
                     (long long)K);
    HC_CU(cudaEventCreateWithFlags(&S.free_ev, cudaEventDisableTiming), "adjoint event");
  }
  // the adjoint iterations' stream
  struct Stream {
    cudaStream_t s = nullptr;
    cudaEvent_t rep = nullptr;
    ~Stream() {
      if (s) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
      }
      if (rep) cudaEventDestroy(rep);
    }
  } rs;
  HC_CU(cudaStreamCreateWithFlags(&rs.s, cudaStreamNonBlocking), "adjoint stream");
  HC_CU(cudaEventCreateWithFlags(&rs.rep, cudaEventDisableTiming), "adjoint event");
  const cudaStream_t sr = rs.s;
  // k_adj_save is part of the graphs while the view's slot pointers are set
  struct SlotGuard {
    hc_ctx* c;
    ~SlotGuard() {
      c->v.adj_sh = c->v.adj_sqx = c->v.adj_sqy = nullptr;
      c->v.adj_smask = nullptr;
      c->graph_iters = 0;
      c->points_hook = nullptr;
      c->points_hook_arg = nullptr;
    }
  } guard{c};
  v.adj_sh = sets[0].h.as<double>();
  v.adj_sqx = sets[0].qx.as<double>();
  v.adj_sqy = sets[0].qy.as<double>();
  v.adj_smask = sets[0].mask.as<uint8_t>();
  c->graph_iters = 0;
  std::vector<Checkpoint> cps((size_t)snaps + 1);  // + the state at the end
  for (auto& cp : cps) HC_TRY(save_state(c, cp, true));
  Revolve rv;
  rv.c = c;
  rv.n = n;
  rv.K = K;
  rv.m = nseg;
  rv.slots = &cps;
  rv.slot_of.assign((size_t)nseg + 1, -1);
  for (int k = snaps - 1; k >= 1; k--) rv.free_slots.push_back(k);
  rv.slot_of[0] = 0;
  // the snapshots of the first sweep: the split points down the right spine
  std::vector<char> first((size_t)nseg + 1, 0);
  {
    int64_t a = 0;
    int sl = snaps - 1;
    while (nseg - a > 1 && sl > 0) {
      a = split_point(a, nseg, sl);
      first[(size_t)a] = 1;
      sl--;
    }
  }
  // ---------------- forward, recording time steps and Q, keeping the
  // first sweep's snapshots
  Dev dt;
  HC_CU(dmalloc(dt, (size_t)n * HC_ADJ_REC * 8), "adjoint record");
  HC_TRY(ctx_pull(c));
  const double cycle0 = c->hdev->s.cycle, time1_0 = c->hdev->s.time_1;
  HC_TRY(adj_mode(c, dt.as<double>(), n, 1, 0));  // no saves in the forward run
  std::vector<hc_step_record> rec((size_t)n);
  const auto t_fwd = std::chrono::steady_clock::now();
  HC_TRY(save_state(c, cps[0], false));
  int64_t done_all = 0;
  for (int64_t g = 0; g < nseg; g++) {
    if (g > 0 && first[(size_t)g]) HC_TRY(rv.keep(g));
    const int64_t len = std::min<int64_t>(K, n - g * K);
    int64_t done = 0;
    HC_TRY(hc_run(c, len, 0, rec.data() + g * K, &done));
    done_all += done;
    if (done != len) {
      adj_mode(c, nullptr, 0, 0, 0);
      return hc_fail(c, HC_ERR_STATE, "the run ended (maxcycle) after %lld of %lld iterations",
                     (long long)done_all, (long long)n);
    }
  }
  HC_TRY(save_state(c, cps[(size_t)snaps], false));  // the end, where the model is left
  HC_CU(cudaStreamSynchronize(s), "adjoint forward");
  const double ms_fwd = ms_since(t_fwd);
  std::vector<double> arec((size_t)n * HC_ADJ_REC);
  HC_CU(cudaMemcpy(arec.data(), dt.p, arec.size() * 8, cudaMemcpyDeviceToHost), "adjoint record");
  // loss and dL/dQ per iteration
  std::vector<int64_t> at;
  samples_of(rec, cycle0, &at);
  const int64_t S = std::min<int64_t>((int64_t)at.size(), n_target);
  std::vector<double> gQ((size_t)n, 0.0);
  double L = 0;
  for (int64_t k = 0; k < S; k++) {
    const double d = rec[(size_t)at[(size_t)k]].waterOut - q_target[k];
    L += d * d / (double)S;
    gQ[(size_t)at[(size_t)k]] = 2 * d / (double)S;
  }
  if (loss) *loss = L;
  // ---------------- reverse
  const auto t_rev = std::chrono::steady_clock::now();
  Dev lam, mux, muy, lamd, p0x, p0y, p1x, p1y, pe0x, pe0y, pe1x, pe1y, gx, gy, gn, ge, gj, pflag;
  if (dmalloc(pflag, N2) || dmalloc(lam, N2 * 8) || dmalloc(mux, N2 * 8) || dmalloc(muy, N2 * 8) ||
      dmalloc(lamd, N2 * 8) || dmalloc(p0x, N2 * 8) || dmalloc(p0y, N2 * 8) ||
      dmalloc(p1x, N2 * 8) || dmalloc(p1y, N2 * 8) || dmalloc(pe0x, N2 * 8) ||
      dmalloc(pe0y, N2 * 8) || dmalloc(pe1x, N2 * 8) || dmalloc(pe1y, N2 * 8) ||
      dmalloc(gx, N2 * 8) || dmalloc(gy, N2 * 8) || dmalloc(gn, N2 * 8) ||
      dmalloc(ge, N2 * 8) || dmalloc(gj, (size_t)n * (HC_MAX_RF + 1) * 8)) {
    adj_mode(c, nullptr, 0, 0, 0);
    return hc_fail(c, HC_ERR_NOMEM, "adjoint: out of device memory");
  }
  for (Dev* d : {&lam, &mux, &muy, &lamd, &p0x, &p0y, &p1x, &p1y, &pe0x, &pe0y, &pe1x, &pe1y,
                 &gx, &gy, &gn, &ge})
    cudaMemsetAsync(d->p, 0, N2 * 8, sr);
  cudaMemsetAsync(gj.p, 0, (size_t)n * (HC_MAX_RF + 1) * 8, sr);
  cudaMemsetAsync(pflag.p, 0, N2, sr);
  dim3 b(32, 8), gr((v.jmax + 31) / 32, (v.imax + 7) / 8);
  double ms_replay = 0;  // host time in the segments' replays
  // device time of each segment's adjoint iterations (event pairs on sr)
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> kev;
  struct EvGuard {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>>* v;
    ~EvGuard() {
      for (auto& e : *v) {
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
      }
    }
  } evg{&kev};
  // the points logs live until the adjoint iterations that read them ran
  std::vector<std::unique_ptr<PointsLog>> logs;
  int64_t leaves = 0;
  rv.advance = [&](int64_t t0, int64_t t1) -> hc_status {
    HC_TRY(adj_mode(c, dt.as<double>(), n, 2, t0));  // imposed steps, no saves
    int64_t done = 0;
    return hc_run(c, t1 - t0, 0, nullptr, &done);
  };
  rv.leaf = [&](int64_t g) -> hc_status {
    const int64_t t0 = g * K, len = std::min<int64_t>(K, n - t0);
    SlotSet& S = sets[nsets == 2 ? (leaves & 1) : 0];
    leaves++;
    // the replay overwrites the set once the adjoint iterations that read
    // it last are done
    HC_CU(cudaStreamWaitEvent(s, S.free_ev, 0), "adjoint");
    // replay as graph runs; k_adj_save keeps every iteration's state
    HC_TRY(adj_mode(c, dt.as<double>(), n, 2, t0, t0, len, &S));
    logs.emplace_back(new PointsLog());
    PointsLog& pts = *logs.back();
    HC_TRY(pts.add(c, t0));
    c->points_hook = points_hook;
    c->points_hook_arg = &pts;
    int64_t done = 0;
    const auto t_rp = std::chrono::steady_clock::now();
    const hc_status rs_ = hc_run(c, len, 0, nullptr, &done);
    c->points_hook = nullptr;
    c->points_hook_arg = nullptr;
    HC_TRY(rs_);
    ms_replay += ms_since(t_rp);
    HC_TRY(adj_mode(c, dt.as<double>(), n, 2, t0 + len));  // saves off
    double* const sqx = S.qx.as<double>();
    double* const sqy = S.qy.as<double>();
    cudaMemcpyAsync(sqx + (size_t)len * N2, v.qx, N2 * 8, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(sqy + (size_t)len * N2, v.qy, N2 * 8, cudaMemcpyDeviceToDevice, s);
    HC_CU(cudaEventRecord(rs.rep, s), "adjoint");
    HC_CU(cudaStreamWaitEvent(sr, rs.rep, 0), "adjoint");
    cudaEvent_t e0, e1;
    HC_CU(cudaEventCreate(&e0), "adjoint event");
    if (cudaEventCreate(&e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      return hc_fail(c, HC_ERR_CUDA, "adjoint event");
    }
    kev.emplace_back(e0, e1);
    HC_CU(cudaEventRecord(e0, sr), "adjoint");
    // adjoint iterations, last first, on sr
    for (int64_t k = len - 1; k >= 0; k--) {
      const int64_t t = t0 + k;
      const double* r = arec.data() + (size_t)t * HC_ADJ_REC;
      AdjStep st;
      std::memset(&st, 0, sizeof st);
      st.input_dt = r[1];
      st.fdt = r[2];
      st.ts = rec[(size_t)t].time_step;
      st.gQ = gQ[(size_t)t];
      AdjBufs bb;
      bb.h0 = S.h.as<double>() + (size_t)k * N2;
      bb.qx0 = sqx + (size_t)k * N2;
      bb.qy0 = sqy + (size_t)k * N2;
      bb.mask = S.mask.as<uint8_t>() + (size_t)k * N2;
      bb.qx1 = sqx + (size_t)(k + 1) * N2;
      bb.qy1 = sqy + (size_t)(k + 1) * N2;
      bb.point = pts.at(t);
      bb.lam = lam.as<double>();
      bb.mux = mux.as<double>();
      bb.muy = muy.as<double>();
      bb.lamd = lamd.as<double>();
      bb.p0x = p0x.as<double>();
      bb.p0y = p0y.as<double>();
      bb.p1x = p1x.as<double>();
      bb.p1y = p1y.as<double>();
      bb.pe0x = pe0x.as<double>();
      bb.pe0y = pe0y.as<double>();
      bb.gx = gx.as<double>();
      bb.gy = gy.as<double>();
      bb.pe1x = pe1x.as<double>();
      bb.pe1y = pe1y.as<double>();
      bb.gn = gn.as<double>();
      bb.ge = ge.as<double>();
      bb.pflag = pflag.as<uint8_t>();
      bb.gj = gj.as<double>() + (size_t)t * (HC_MAX_RF + 1);
      const double* na = pts.nact_at(t);
      const double* ct = pts.cnt_at(t);
      for (int z = 0; z <= v.p.rfnum && z <= HC_MAX_RF; z++) {
        double a = (r[3 + z] * na[z]) / (ct[z]) * st.input_dt;
        double da = na[z] / ct[z] * st.input_dt;
        if (a > v.p.ERODEFACTOR) a = v.p.ERODEFACTOR, da = 0;
        st.amt[z] = a;
        st.damt[z] = da;
      }
      k_adj_depth<<<gr, b, 0, sr>>>(v, bb, st);
      k_adj_flow_c<<<c->sms * 4, 256, 0, sr>>>(v, bb, st);
      k_adj_gather<<<gr, b, 0, sr>>>(v, bb, st);
    }
    HC_CU(cudaGetLastError(), "adjoint kernels");
    HC_CU(cudaEventRecord(e1, sr), "adjoint");
    HC_CU(cudaEventRecord(S.free_ev, sr), "adjoint");
    return HC_OK;
  };
  HC_TRY(rv.reverse(0, nseg, snaps - 1));
  HC_CU(cudaStreamSynchronize(sr), "adjoint");
  HC_CU(cudaStreamSynchronize(s), "adjoint");
  const double ms_rev = ms_since(t_rev);
  double ms_kernels = 0;
  for (auto& e : kev) {
    float f = 0;
    HC_CU(cudaEventElapsedTime(&f, e.first, e.second), "adjoint event");
    ms_kernels += f;
  }
  // ---------------- results
  if (grad_n) HC_CU(cudaMemcpy(grad_n, gn.p, N2 * 8, cudaMemcpyDeviceToHost), "adjoint gradient");
  if (grad_elev) HC_CU(cudaMemcpy(grad_elev, ge.p, N2 * 8, cudaMemcpyDeviceToHost), "adjoint gradient");
  if (grad_rain) {
    int rows = 0, cols = 0;
    const float* rain = ctx_rain(c, &rows, &cols);
    std::fill(grad_rain, grad_rain + (size_t)rows * cols, 0.0);
    std::vector<double> gjh((size_t)n * (HC_MAX_RF + 1));
    HC_CU(cudaMemcpy(gjh.data(), gj.p, gjh.size() * 8, cudaMemcpyDeviceToHost), "adjoint gradient");
    // j used by iteration t was made by the iteration before it (time_1,
    // cycle of that calchydrograph); the first by the state before the run
    int max_row = (int)time1_0;
    for (int64_t t = 0; t < n; t++)
      max_row = std::max(max_row, (int)arec[(size_t)t * HC_ADJ_REC + HC_ADJ_T1]);
    const int nsteps = max_row + 1, rf = v.p.rfnum;
    std::vector<double> dold((size_t)nsteps * (rf + 1) * rows), dnew(dold.size());
    host_topmodel_tangent(&v.p, rain, rows, cols, nsteps, dold.data(), dnew.data());
    for (int64_t t = 0; t < n; t++) {
      const double t1 = (t == 0) ? time1_0 : arec[(size_t)(t - 1) * HC_ADJ_REC + HC_ADJ_T1];
      const double cyc = (t == 0) ? cycle0 : arec[(size_t)(t - 1) * HC_ADJ_REC + HC_ADJ_T1 + 1];
      const double w = (2 - (t1 - cyc)) / 2;
      const int row = (int)t1;
      for (int z = 1; z <= rf && z - 1 < cols; z++) {
        const double g = gjh[(size_t)t * (HC_MAX_RF + 1) + z];
        if (g == 0) continue;
        const double* ro = dold.data() + ((size_t)row * (rf + 1) + z) * rows;
        const double* rn = dnew.data() + ((size_t)row * (rf + 1) + z) * rows;
        for (int k = 0; k < rows; k++) grad_rain[(size_t)k * cols + (z - 1)] += g * (ro[k] * (1 - w) + rn[k] * w);
      }
    }
  }
  // leave the model where the forward run ended
  HC_TRY(load_state(c, cps[(size_t)snaps]));
  HC_TRY(adj_mode(c, nullptr, 0, 0, 0));
  if (ms) {
    ms[0] = ms_fwd;
    ms[1] = ms_rev;
    ms[2] = ms_since(t_all);
    ms[3] = (double)K;
    ms[4] = (double)snaps;
    ms[5] = (double)rv.advances;
    ms[6] = ms_replay;
    ms[7] = ms_kernels;
  }
  return HC_OK;
}

void launch_adj_save(hc_ctx* c) {
  k_adj_save<<<152 * 4, 256, 0, c->cs>>>(c->v, c->dev);
  count_launch(c, 1);
}
