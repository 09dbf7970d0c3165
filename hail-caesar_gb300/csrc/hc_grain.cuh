// Grain-store members of the reference on the device record layout:
// sort_active :3874-3947, sand_fraction :3985-4009, d50 :4038-4075,
// slide_GS :4077-4171, mean_ws_elev :4011-4036.
//
// A cell's record lives in its own slot (grain_at, strata_at in
// hc_internal.cuh); index[cell] == -9999 means "no record" exactly as in the
// reference.
#pragma once
#include "hc_internal.cuh"

HC_DEV double& GRN(const hc_view& c, size_t cell, int n) { return grain_at(c, cell, n); }
HC_DEV double& STR(const hc_view& c, size_t cell, int z, int n) {
  return strata_at(c, cell, z, n);
}

// addGS for contexts that run in the reference's serial order (one thread):
// the record gets the next row number.
HC_DEV void addGS_serial(const hc_view& c, hc_dev* d, size_t cell) {
  d->grain_tot++;
  c.index[cell] = d->grain_tot;
  grain_record_init(c, cell, c.elev[cell], c.bed[cell]);
}

HC_DEV void sort_active_dev(const hc_view& c, hc_dev* d, size_t cell, bool may_alloc) {
  if (c.index[cell] == -9999) {
    if (may_alloc) {
      addGS_serial(c, d, cell);
    } else {
      d->err_code = 201;  // allocation outside serial context (cannot happen)
      d->pause |= HC_PAUSE_ERROR;
      return;
    }
  }
  const double active = c.p.active;
  // total of the record decides between "deposit a stratum", "eat into the
  // stratum below" and nothing.  A float sum with a bound on its error
  // decides the two tests; the FP64 sum of the reference (needed anyway when
  // a stratum moves) is formed only when the float sum is too close to call.
  double g[HC_G + 1];
  float sf = 0.0f, af = 0.0f;
  for (int n = 0; n <= HC_G; n++) {
    g[n] = GRN(c, cell, n);
    const float f = approx_f(g[n]);
    sf += f;
    af += fabsf(f);
  }
  const float tol = 1e-5f * af + 1e-30f;
  const float hi = c.act_hi, lo = c.act_lo;
  int dep = (sf > hi + tol) ? 1 : ((sf < hi - tol) ? -1 : 0);
  int ero = (sf < lo - tol) ? 1 : ((sf > lo + tol) ? -1 : 0);
  if (dep == -1 && ero == -1) return;
  double total = 0.0;
  for (int n = 0; n <= HC_G; n++) total += g[n];
  if (total > (active * 1.5)) {
    for (int z = 9; z >= 1; z--)
      for (int n = 0; n <= HC_G - 2; n++) STR(c, cell, z, n) = STR(c, cell, z - 1, n);
    double coeff = active / total;
    for (int n = 1; n <= HC_G - 1; n++) {
      if (g[n] > 0.0) {
        double amount = coeff * (g[n]);
        STR(c, cell, 0, n - 1) = amount;
        GRN(c, cell, n) = g[n] - amount;
      }
    }
  }
  if (total < (active / 4)) {
    for (int n = 1; n <= HC_G - 1; n++) GRN(c, cell, n) += STR(c, cell, 0, n - 1);
    for (int z = 0; z <= 8; z++)
      for (int n = 0; n <= HC_G - 2; n++) STR(c, cell, z, n) = STR(c, cell, z + 1, n);
    for (int n = 1; n <= HC_G - 1; n++) STR(c, cell, 9, n - 1) = active * c.p.dprop[n];
  }
}

HC_DEV double sand_fraction_dev(const hc_view& c, size_t cell) {
  double at = 0, st = 0;
  for (int n = 1; n <= HC_G; n++) at += GRN(c, cell, n);
  for (int n = 1; n <= 2; n++) st += GRN(c, cell, n);
  if (at < 0.0001) return 0.0;
  return st / at;
}

HC_DEV double d50_dev(const hc_view& c, size_t cell) {
  double at = 0, mx = 0, mn = 0;
  double cum[HC_G + 1];
  cum[0] = 0;
  for (int n = 1; n <= HC_G; n++) {
    at += GRN(c, cell, n);
    cum[n] = at;
  }
  int i = 1;
  while (i <= 9 && cum[i] < (at * 0.5)) i++;
  if (i <= 9) {
    mn = c.dlog[(i == 1) ? 1 : i - 1];
    mx = c.dlog[i];
  }
  double cum_i = (i <= HC_G) ? cum[i] : 0.0;
  double Dfifty = exp(mx - ((mx - mn) * ((cum_i - (at * 0.5)) / (cum_i - cum[i - 1]))));
  if (at < 0.0000001) Dfifty = 0;
  return Dfifty;
}

// slide_GS(x,y -> x2,y2, amount).  may_alloc: the caller runs in serial order
// (case 3 allocates the receiver's record).
HC_DEV void slide_GS_dev(const hc_view& c, hc_dev* d, size_t a, double amount, size_t b,
                         bool may_alloc) {
  const double* dprop = c.p.dprop;
  double total = 0;
  const bool ha = c.index[a] != -9999, hb = c.index[b] != -9999;
  if (ha && hb) {
    for (int n = 1; n <= HC_G - 1; n++)
      if (GRN(c, a, n) > 0) total += GRN(c, a, n);
    if (amount > total) {
      for (int n = 1; n <= HC_G - 1; n++) GRN(c, b, n) += (amount - total) * dprop[n];
      amount = total;
    }
    if (total > 0) {
      // grain/total for the nine fractions: one prepared divisor, then the
      // exact quotient of each (ddiv_by)
      const hc_divisor td = ddiv_prep(total);
      for (int n = 1; n <= HC_G - 1; n++) {
        const double ga = GRN(c, a, n);
        double t = amount * ddiv_by(ga, td);
        GRN(c, b, n) += t;
        double na = ga - t;
        if (na < 0) na = 0;
        GRN(c, a, n) = na;
      }
    }
    sort_active_dev(c, d, a, may_alloc);
    sort_active_dev(c, d, b, may_alloc);
    return;
  }
  if (!ha && hb) {
    for (int n = 1; n <= HC_G - 1; n++) GRN(c, b, n) += (amount)*dprop[n];
    sort_active_dev(c, d, b, may_alloc);
    return;
  }
  if (ha && !hb) {
    if (!may_alloc) {
      d->err_code = 202;
      d->pause |= HC_PAUSE_ERROR;
      return;
    }
    addGS_serial(c, d, b);
    if (amount > c.p.active) {
      for (int n = 1; n <= HC_G - 1; n++) GRN(c, b, n) += amount * dprop[n];
      amount = c.p.active;
    }
    for (int n = 1; n <= HC_G - 1; n++)
      if (GRN(c, a, n) > 0) total += GRN(c, a, n);
    if (total > 0) {
      const hc_divisor td = ddiv_prep(total);
      for (int n = 1; n <= HC_G - 1; n++) {
        const double ga = GRN(c, a, n);
        const double t = amount * ddiv_by(ga, td);
        GRN(c, b, n) += t;
        double na = ga;
        if (na > 0.0001) na -= t;
        if (na < 0) na = 0;
        GRN(c, a, n) = na;
      }
    }
    sort_active_dev(c, d, a, may_alloc);
    sort_active_dev(c, d, b, may_alloc);
    return;
  }
}

HC_DEV double mean_ws_elev_dev(const hc_view& c, int x, int y) {
  const int dX[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1};
  const int dY[9] = {0, -1, -1, 0, 1, 1, 1, 0, -1};
  double et = 0;
  int cnt = 0;
  for (int dir = 1; dir <= 8; dir++) {
    size_t q = (size_t)(x + dX[dir]) * c.W + (y + dY[dir]);
    if (c.h[q] > c.p.water_depth_erosion_threshold) {
      et += c.h[q] + c.elev[q];
      cnt++;
    }
  }
  if (cnt > 0) {
    et /= cnt;
    return et;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// grain records held in registers (the apply walkers, the slide_3 replay)
// ---------------------------------------------------------------------------
// A cell as the apply walkers hold it.
struct ApplyRow {
  double g[HC_G + 1];  // grain record, planes 0..HC_G
  double elev, h, bed, edge;
  int idx;             // index[] (-9999: no record)
  bool dirty;          // g[1..9] or elev changed
};

__device__ __forceinline__ void row_load(const hc_view& c, size_t cell, size_t ecell,
                                         ApplyRow& r) {
#pragma unroll
  for (int n = 0; n <= HC_G; n++) r.g[n] = GRN(c, cell, n);
  r.elev = c.elev[cell];
  r.h = c.h[cell];
  r.bed = c.bed[cell];
  r.edge = c.edge[ecell];
  r.idx = c.index[cell];
  r.dirty = false;
}

__device__ __forceinline__ void row_store(const hc_view& c, size_t cell, const ApplyRow& r) {
  if (!r.dirty) return;
#pragma unroll
  for (int n = 1; n <= HC_G - 1; n++) GRN(c, cell, n) = r.g[n];
  c.elev[cell] = r.elev;
}

// sort_active on a held row; the strata stay in memory (they move only when
// the record crosses a threshold).  Same decisions as sort_active_dev.
static __device__ void sort_active_row(const hc_view& c, hc_dev* d, size_t cell, ApplyRow& r) {
  if (r.idx == -9999) {
    d->err_code = 201;  // records were allocated before the pass (cannot happen)
    d->pause |= HC_PAUSE_ERROR;
    return;
  }
  const double active = c.p.active;
  float sf = 0.0f, af = 0.0f;
#pragma unroll
  for (int n = 0; n <= HC_G; n++) {
    const float f = approx_f(r.g[n]);
    sf += f;
    af += fabsf(f);
  }
  const float tol = 1e-5f * af + 1e-30f;
  const float hi = c.act_hi, lo = c.act_lo;
  const int dep = (sf > hi + tol) ? 1 : ((sf < hi - tol) ? -1 : 0);
  const int ero = (sf < lo - tol) ? 1 : ((sf > lo + tol) ? -1 : 0);
  if (dep == -1 && ero == -1) return;
  double total = 0.0;
#pragma unroll
  for (int n = 0; n <= HC_G; n++) total += r.g[n];
  if (total > (active * 1.5)) {
    for (int z = 9; z >= 1; z--)
      for (int n = 0; n <= HC_G - 2; n++) STR(c, cell, z, n) = STR(c, cell, z - 1, n);
    const double coeff = active / total;
#pragma unroll
    for (int n = 1; n <= HC_G - 1; n++) {
      if (r.g[n] > 0.0) {
        const double amount = coeff * (r.g[n]);
        STR(c, cell, 0, n - 1) = amount;
        r.g[n] = r.g[n] - amount;
      }
    }
    r.dirty = true;
  }
  if (total < (active / 4)) {
#pragma unroll
    for (int n = 1; n <= HC_G - 1; n++) r.g[n] += STR(c, cell, 0, n - 1);
    for (int z = 0; z <= 8; z++)
      for (int n = 0; n <= HC_G - 2; n++) STR(c, cell, z, n) = STR(c, cell, z + 1, n);
    for (int n = 1; n <= HC_G - 1; n++) STR(c, cell, 9, n - 1) = active * c.p.dprop[n];
    r.dirty = true;
  }
}

// slide_GS(a -> b, amount) on held rows (records exist: allocated before the
// pass).  Same arithmetic as slide_GS_dev.
// The sum of A's positive fractions, in order: slide_GS's `total`.
__device__ __forceinline__ double positive_total(const ApplyRow& A) {
  double total = 0;
#pragma unroll
  for (int n = 1; n <= HC_G - 1; n++)
    if (dgt0(A.g[n])) total += A.g[n];
  return total;
}

// total_a: positive_total(A), which the caller may have formed ahead (the
// sum is a chain of nine dependent FP64 additions)
static __device__ void slide_GS_rows(const hc_view& c, hc_dev* d, size_t a, ApplyRow& A, double amount,
                              size_t b, ApplyRow& B, double total_a) {
  const double* dprop = c.p.dprop;
  const bool ha = A.idx != -9999, hb = B.idx != -9999;
  if (ha && hb) {
    const double total = total_a;
    if (dgt(amount, total)) {
#pragma unroll
      for (int n = 1; n <= HC_G - 1; n++) B.g[n] += (amount - total) * dprop[n];
      amount = total;
    }
    if (dgt0(total)) {
      const hc_divisor td = ddiv_prep(total);
#pragma unroll
      for (int n = 1; n <= HC_G - 1; n++) {
        const double ga = A.g[n];
        const double t = amount * ddiv_by(ga, td);
        B.g[n] += t;
        double na = ga - t;
        if (dlt0(na)) na = 0;
        A.g[n] = na;
      }
    }
    A.dirty = B.dirty = true;
    sort_active_row(c, d, a, A);
    sort_active_row(c, d, b, B);
    return;
  }
  if (!ha && hb) {
#pragma unroll
    for (int n = 1; n <= HC_G - 1; n++) B.g[n] += (amount)*dprop[n];
    B.dirty = true;
    sort_active_row(c, d, b, B);
    return;
  }
  if (ha && !hb) {
    d->err_code = 202;  // receiver without a record outside a serial context
    d->pause |= HC_PAUSE_ERROR;
  }
}
