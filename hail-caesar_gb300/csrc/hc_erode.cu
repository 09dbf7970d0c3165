// erode(mult) :4211-4845 ("erodedepo"), with call_erosion :2277-2294.
//
// Structure on the device:
//   k_erode_begin    time_step *= 1.5 (:4219), open the retry loop (a direct
//                    call; an iteration's k_control does this itself)
//   k_entrain_tau, k_entrain  the entrainment pass (:4236-4548): shear stress
//                    per cell, then the transport of the cells with tau > 0;
//                    its last block evaluates the retry test (:4550-4565)
//   k_alloc_*        grain records requested during the pass get the
//                    reference's row numbers in the reference's serial order
//   k_apply_*        the gather-apply pass with the in-line +/-x lateral
//                    erosion (:4570-4682) and the +/-y lateral pass
//                    (:4684-4747), walked in order along independent chains
//   k_edge_out       sediment leaving the four edges (:4750-4841), then
//                    erode_mult / erode_call of call_erosion
//
// Allocation order.  The reference numbers grain records (addGS) in the order
// its serial loop asks for them: during the entrainment pass a cell asks for
// itself (before its transport) and for wet neighbours it sends bedload to
// (directions 1,3,5,7, after its transport).  Each request here is keyed by
// (loop position of the asking cell) * 5 + (0 self, 1..4 neighbour); a
// cell's record is numbered by the smallest key that asked for it, which is
// exactly the request that allocated it in the serial loop.  Record contents
// do not depend on the number (elevation and bedrock are not changed by the
// pass before a record is made), so the pass itself runs in parallel.

#include "hc_grain.cuh"

#include <math.h>

namespace {

constexpr double kG = 9.81;
__constant__ int kDXc[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1};
__constant__ int kDYc[9] = {0, -1, -1, 0, 1, 1, 1, 0, -1};

// plane of the outgoing-flux arrays: dir 0 su (p=1), 1 sr (p=3), 2 sd (p=5), 3 sl (p=7)
__device__ __forceinline__ double& SF(const hc_view& c, int dir, int n, size_t cell) {
  return c.sflux[((size_t)dir * 10 + n) * c.N2 + cell];
}
__device__ __forceinline__ size_t EX(const hc_view& c, int x, int y) {
  return (size_t)x * (c.jmax + 1) + y;
}

// The Einstein transport of one fraction (:4398-4405) and the bedrock
// rescaling's division, out of line: the fraction loop is unrolled, and with
// their integer-pipe divisions and cube inlined nine times over the
// transport kernel's code would be several times larger.
static __device__ __noinline__ double einstein_td(double mts, double einA, hc_divisor Bd,
                                                  hc_divisor einSd, hc_divisor dxd) {
  const double x = ddiv_by(einA, Bd);
  return ddiv_by(ddiv_by(mts * (40 * icube_rn(ddiv_rn(1.0, x))), einSd), dxd);
}
static __device__ __noinline__ double ddiv_rn_entrain(double a, double b) { return ddiv_rn(a, b); }

// blocks of 128 threads of the transport kernel (grid-stride over its
// list): 1216 on large grids, fewer on small ones, whose lists are short and
// whose idle blocks would only cost dispatch (ensembles of small members run
// many such launches side by side)
static unsigned entrain_blocks(size_t N2) {
  return (unsigned)std::min<size_t>(152 * 8, std::max<size_t>(16, N2 / 1024));
}

__global__ void k_erode_begin(const hc_view c, hc_dev* d, int gated, double mult_override) {
  if (gated) {
    if (!(d->it_active && d->do_erode)) return;
  } else {
    d->do_erode = 1;
    d->it_active = 1;
    d->rest_active = 1;
  }
  d->s.time_step = d->s.time_step * 1.5;
  d->mult = (mult_override >= 0) ? mult_override : d->s.erode_mult;
  d->erode_retry = 1;
  d->erode_passes = 0;
  d->tempbmax_bits = 0;
}

// ---------------------------------------------------------------------------
// entrainment pass
// ---------------------------------------------------------------------------
// Two kernels.  k_entrain_tau, one thread per cell, clears the pass's
// outputs (the 40 outgoing-flux entries only where the last transport wrote
// some, sdirty: clearing zeros was 320 B of writes per masked cell and
// pass), makes the records of cells that ask for one, sums the squared
// velocities and slopes, and lists the cells with flow (qtot > 0; one
// atomic per warp).  k_entrain computes the shear stress and the transport
// of the listed cells only, so its warps are full: in a storm, a third or
// less of the lanes of a row of cells has flow, and these terms (pow, the
// Einstein or Wilcock sums) are FP64-pipe bound.
__global__ void __launch_bounds__(128) k_entrain_tau(const hc_view c, hc_dev* d) {
  if (!(d->it_active && d->erode_retry)) return;
  const hc_params& p = c.p;
  const int jy = 1 + blockIdx.x * blockDim.x + threadIdx.x;  // column y
  const int ix = 1 + blockIdx.y * blockDim.y + threadIdx.y;  // row x
  const size_t W = c.W, N2 = c.N2;
  const double thr = p.water_depth_erosion_threshold;
  bool listed = false;
  size_t cell = 0;
  double qtot = 0, slopetot = 0;
  if (ix <= c.imax && jy <= c.jmax - 1) {
    cell = (size_t)ix * W + jy;
    if (c.mask[cell]) {
      c.vel[cell] = 0;
      c.tau[cell] = 0;
      if (c.sdirty[cell]) {
        for (int n = 0; n < HC_G; n++) {
          SF(c, 0, n, cell) = 0;
          SF(c, 1, n, cell) = 0;
          SF(c, 2, n, cell) = 0;
          SF(c, 3, n, cell) = 0;
        }
        c.sdirty[cell] = 0;
      }
      c.ss[cell] = 0;
      const double h = c.h[cell];
      if (dgt(h, thr)) {
        const double e0 = c.elev[cell];
        const unsigned long long pos = (unsigned long long)jy * (c.imax + 2) + ix;
        if (c.index[cell] == -9999) {  // addGS(x, y)
          grain_record_init(c, cell, e0, c.bed[cell]);
          c.index[cell] = -2;  // record made, row number pending
          atomicMin(&c.alloc_key[cell], pos * 5);
          d->alloc_count = 1;
        }
        double vel = 0;
        for (int k = 0; k < 4; k++) {
          const int pp = 1 + 2 * k;
          const int x2 = ix + kDXc[pp], y2 = jy + kDYc[pp];
          const size_t nb = (size_t)x2 * W + y2;
          if (dgt(c.h[nb], thr)) {
            const double vdir = c.vd[(size_t)k * N2 + cell];
            if (dgt0(vdir)) {
              vel = vdir;
              if (dgt(vel, p.max_vel)) vel = p.max_vel;
              qtot += (vel * vel);
              slopetot += ddiv_by(e0 - c.elev[nb], c.dxd) * vel;
            }
          }
        }
        // the shear stress itself (:4316-4333: sqrt, pow(h, -0.33)) is
        // evaluated by k_entrain for the listed cells, whose warps are full
        listed = dgt0(qtot);
      }
    }
  }
  // blockDim.x == 32: a warp is one run of columns
  const unsigned lane = threadIdx.x;
  const unsigned b = __ballot_sync(0xffffffffu, listed);
  if (b) {
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(&d->ent_n, (unsigned)__popc(b));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (listed) {
      const unsigned k = base + __popc(b & ((1u << lane) - 1));
      c.ent_list[k] = (uint32_t)cell;
      c.ent_qs[2 * (size_t)k] = qtot;
      c.ent_qs[2 * (size_t)k + 1] = slopetot;
    }
  }
}

// The shear stress (:4316-4333) and the transport (:4388-4548) of one
// listed cell (qtot > 0); returns temptot1.
__device__ double entrain_cell(const hc_view& c, hc_dev* d, size_t cell, double mult,
                               double ts, double qtot, double slopetot) {
  const hc_params& p = c.p;
  const size_t W = c.W, N2 = c.N2;
  const int ix = (int)(cell / W), jy = (int)(cell % W);
  const double thr = p.water_depth_erosion_threshold;
  const double h = c.h[cell];
  double tau;
  {
    double vel = isqrt_rn(qtot);
    c.vel[cell] = vel;
    if (dgt(vel, p.max_vel)) vel = p.max_vel;
    const double n_man = p.spatially_var_mannings ? c.man[cell] : p.mannings;
    const double ci = kG * (n_man * n_man) * pow(h, -0.33);
    if (dgt0(slopetot)) slopetot = 0;
    tau = 1000 * ci * vel * vel * (1 + (1 * ddiv_rn(slopetot, vel)));
    c.tau[cell] = tau;
    if (!dgt0(tau)) return 0;  // no transport from this cell
  }
  const double rho = 1000.0;
  const double e0 = c.elev[cell];
  const unsigned long long pos = (unsigned long long)jy * (c.imax + 2) + ix;
  // the direction weights of the velocity pass (:4250-4289), again
  double temptot2 = 0, veltot = 0;
  double tempdir[4] = {0, 0, 0, 0};
  const double edge0 = c.edge[EX(c, ix, jy)];
  for (int k = 0; k < 4; k++) {
    const int pp = 1 + 2 * k;
    const int x2 = ix + kDXc[pp], y2 = jy + kDYc[pp];
    const size_t nb = (size_t)x2 * W + y2;
    if (dgt(c.h[nb], thr)) {
      const double edge2 = c.edge[EX(c, x2, y2)];
      if (dgt(edge0, edge2)) temptot2 += (edge0 - edge2);
      const double vdir = c.vd[(size_t)k * N2 + cell];
      if (dgt0(vdir)) {
        double vel = vdir;
        if (dgt(vel, p.max_vel)) vel = p.max_vel;
        tempdir[k] = vel * vel;
        veltot += tempdir[k];
      }
    }
  }
  double temp_dist[HC_G] = {0};
  double d_50 = 0, Fs = 0, graintot = 0;
  if (p.wilcock) {
    d_50 = d50_dev(c, cell);
    if (d_50 < p.d[1]) d_50 = p.d[1];
    Fs = sand_fraction_dev(c, cell);
    for (int n = 1; n <= HC_G; n++) graintot += GRN(c, cell, n);
  }
  double temptot1 = 0;
  const double mts = mult * ts;
  // Einstein: 1 / ((1650 Di) / (tau/g)); the nine quotients by tau/g
  // share one prepared divisor
  const double Bq = ddiv_rn(tau, kG);
  const hc_divisor Bd = ddiv_prep(Bq);
  for (int n = 1; n <= HC_G - 1; n++) {
    const double Di = p.d[n];
    double td = 0;
    if (p.wilcock) {
      double tau_ri = (0.021 + (0.015 * exp(-20 * Fs))) * (rho * kG * d_50) *
                      pow((Di / d_50), (0.67 / (1 + exp(1.5 - (Di / d_50)))));
      // pow(tau / rho, 0.5): the square root, correctly rounded
      double U_star = isqrt_rn(tau / rho);
      double Fi = GRN(c, cell, n) / graintot;
      double Wi_star;
      if ((tau / tau_ri) < 1.35)
        Wi_star = 0.002 * pow(tau / tau_ri, 7.5);
      else
        Wi_star = 14 * pow(1 - (0.894 / sqrt(tau / tau_ri)), 4.5);
      td = ddiv_by(mts * ((Fi * (U_star * U_star * U_star)) / ((2.65 - 1) * kG)) * Wi_star,
                   c.dxd);
    }
    if (p.einstein) td = einstein_td(mts, c.einA[n], Bd, c.einSd[n], c.dxd);
    if (dgt(td, GRN(c, cell, n))) td = GRN(c, cell, n);
    if (p.isSuspended[n] && n == 1) {
      if (dgt((td + c.vs[cell]) / h, p.Csuspmax)) td = (h * p.Csuspmax) - c.vs[cell];
    }
    if (dlt0(td)) td = 0;
    temp_dist[n] = td;
    temptot1 += td;
  }
  const double bed = c.bed[cell];
  if (!dgt(e0 - temptot1, bed)) {
    double elevdiff = e0 - bed;
    double temptot3 = temptot1;
    temptot1 = 0;
    for (int n = 1; n <= HC_G - 1; n++) {
      if (!dgt(e0, bed)) {
        temp_dist[n] = 0;
      } else {
        temp_dist[n] = elevdiff * ddiv_rn_entrain(temp_dist[n], temptot3);
        if (dlt0(temp_dist[n])) temp_dist[n] = 0;
      }
      temptot1 += temp_dist[n];
    }
    if (dgt(tau, p.bedrock_erosion_threshold)) {
      double amount = pow(p.bedrock_erosion_rate * tau, 1.5) * ts * mult * 0.000000317;
      c.bed[cell] = bed - amount;
      for (int n2 = 1; n2 <= HC_G - 1; n2++) GRN(c, cell, n2) += amount * p.dprop[n2];
    }
  }
  // vegetation terms (:4459-4488) vanish: vegetation is not supported
  // (hc_create rejects vegetation_on) and veg stays zero.
  if (dgt0(temptot1)) {
    c.sdirty[cell] = 1;  // the next pass clears this cell's flux entries
    for (int k = 0; k < 4; k++) {
      const int pp = 1 + 2 * k;
      const int x2 = ix + kDXc[pp], y2 = jy + kDYc[pp];
      const size_t nb = (size_t)x2 * W + y2;
      if (dgt(c.h[nb], thr)) {
        if (c.index[nb] < 1) {  // no final row number yet: ask
          atomicMin(&c.alloc_key[nb], pos * 5 + 1 + k);
          d->alloc_count = 1;
        }
        double factor = 0;
        if (dgt0(c.vd[(size_t)k * N2 + cell])) factor += ddiv_rn(0.75 * tempdir[k], veltot);
        const double edge2 = c.edge[EX(c, x2, y2)];
        if (dgt(edge0, edge2)) factor += 0.25 * ddiv_rn(edge0 - edge2, temptot2);
        for (int n = 1; n <= HC_G - 1; n++) {
          if (dgt0(temp_dist[n])) {
            if (n == 1 && p.isSuspended[n]) {
              c.ss[cell] = temp_dist[n];
            } else {
              SF(c, k, n, cell) = temp_dist[n] * factor;
            }
          }
        }
      }
    }
  }
  return temptot1;
}

__global__ void __launch_bounds__(128) k_entrain(const hc_view c, hc_dev* d, int max_passes,
                                                  cudaGraphConditionalHandle next, int has_next) {
  __shared__ double wmax[4];
  __shared__ bool last;
  if (!(d->it_active && d->erode_retry)) return;
  const hc_params& p = c.p;
  const double mult = d->mult, ts = d->s.time_step;
  const unsigned n_list = *(volatile unsigned*)&d->ent_n;
  double tb = 0;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n_list;
       k += gridDim.x * blockDim.x)
    tb = smax(tb, entrain_cell(c, d, c.ent_list[k], mult, ts, c.ent_qs[2 * (size_t)k],
                               c.ent_qs[2 * (size_t)k + 1]));
  // tempbmax: max over the pass (warp shuffle, block, grid via last block)
  for (int o = 16; o > 0; o >>= 1) tb = smax(tb, __shfl_xor_sync(0xffffffffu, tb, o));
  const int t = threadIdx.x;
  if ((t & 31) == 0) wmax[t >> 5] = tb;
  __syncthreads();
  if (t == 0) {
    double b = 0;
    for (int w = 0; w < (int)blockDim.x / 32; w++) b = smax(b, wmax[w]);
    if (b > 0) atomic_max_pos(&d->tempbmax_bits, b);
    __threadfence();
    last = (atomicAdd(&d->pass_done, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last && t == 0) {
    __threadfence();
    const double tempbmax = __longlong_as_double((long long)atomicExch(&d->tempbmax_bits, 0ull));
    d->pass_done = 0;
    d->ent_n = 0;
    d->erode_passes++;
    const double EF = p.ERODEFACTOR;
    if (tempbmax > EF) {
      d->s.time_step *= (EF / tempbmax) * 0.5;
      d->erode_retry = 1;
      if (max_passes > 0 && d->erode_passes >= max_passes) {
        d->pause |= HC_PAUSE_ERODE;
        d->rest_active = 0;
      }
    } else {
      d->erode_retry = 0;
    }
    if (has_next) {
      cudaGraphSetConditional(next, d->erode_retry ? 1u : 0u);
      if (d->erode_retry) d->body_kernels += 5;  // the next pass's kernels
    }
    d->s.tempbmax = tempbmax;  // tempbmax of the last pass
  }
}

// ---------------------------------------------------------------------------
// row numbers for the records requested in the pass just run
// ---------------------------------------------------------------------------
// Mark: for every requested cell set bit (key % 5) of position key / 5 and
// make the record if the cell did not make it itself.
__global__ void k_alloc_mark(const hc_view c, hc_dev* d, uint32_t* bits) {
  if (!d->alloc_count) return;
  const size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= c.N2) return;
  const unsigned long long key = c.alloc_key[cell];
  if (key == ~0ull) return;
  c.alloc_key[cell] = ~0ull;
  if (c.index[cell] == -9999) {
    grain_record_init(c, cell, c.elev[cell], c.bed[cell]);
    c.index[cell] = -2;
  }
  const unsigned long long P = key / 5;
  const unsigned sub = (unsigned)(key % 5);
  atomicOr(&bits[P >> 2], (1u << sub) << ((P & 3) * 8));
}

// Per-block counts of requested records (1024 threads x 4 positions); the
// block that finishes last scans them (exclusive, in place) and stores the
// total.
__global__ void __launch_bounds__(1024) k_alloc_count(const hc_view c, hc_dev* d,
                                                      const uint32_t* bits, int32_t* block_sums,
                                                      size_t nwords, int32_t* total_out) {
  __shared__ int ws[32];
  if (!d->alloc_count) return;
  const size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int cnt = (w < nwords) ? __popc(bits[w]) : 0;
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < (int)blockDim.x / 32; k++) s += ws[k];
    block_sums[blockIdx.x] = s;
  }
  if (!last_to_arrive(&d->alloc_arrive)) return;
  const int total = scan_block_counts(block_sums, (int)gridDim.x);
  if (threadIdx.x == 0) *total_out = total;
}

// Assign row numbers in key order and clear the bits; the block that
// finishes last adds the new records to the count.
__global__ void __launch_bounds__(1024) k_alloc_assign(const hc_view c, hc_dev* d,
                                                       uint32_t* bits, const int32_t* block_sums,
                                                       size_t nwords, const int32_t* total) {
  __shared__ int ws[32];
  __shared__ int wbase[32];
  if (!d->alloc_count) return;
  const size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t word = (w < nwords) ? bits[w] : 0u;
  int cnt = __popc(word);
  // inclusive warp scan
  int incl = cnt;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < (int)blockDim.x / 32; k++) {
      wbase[k] = s;
      s += ws[k];
    }
  }
  __syncthreads();
  if (word) {
    int r = block_sums[blockIdx.x] + wbase[warp] + incl - cnt;
    const int base = d->grain_tot + 1;
    for (int byte = 0; byte < 4; byte++) {
      const unsigned b = (word >> (byte * 8)) & 0xffu;
      if (!b) continue;
      const unsigned long long P = (unsigned long long)w * 4 + byte;
      const int y = (int)(P / (unsigned long long)(c.imax + 2));
      const int x = (int)(P % (unsigned long long)(c.imax + 2));
      for (int sub = 0; sub < 5; sub++) {
        if (!(b & (1u << sub))) continue;
        int tx = x, ty = y;
        if (sub > 0) {
          const int pp = 2 * sub - 1;
          tx += kDXc[pp];
          ty += kDYc[pp];
        }
        c.index[(size_t)tx * c.W + ty] = base + r;
        r++;
      }
    }
    bits[w] = 0u;
  }
  // every block has read grain_tot and alloc_count when the last arrives
  if (!last_to_arrive(&d->assign_arrive)) return;
  if (threadIdx.x == 0) {
    d->grain_tot += *total;
    d->s.grain_array_tot = d->grain_tot;
    d->alloc_count = 0;
  }
}

// ---------------------------------------------------------------------------
// apply pass :4570-4682 (gather + lateral step along the columns) and the
// +/-y lateral pass :4684-4748
// ---------------------------------------------------------------------------
// The apply passes are sequential in the reference: along a column the
// +/-x lateral step of row x changes rows x-1 and x+1 before row x+1 is
// processed (and along a row for the +/-y pass).  Only cells with bedload
// leaving them (erodetot3 > 0, "lateral cells") take that step, so a column
// splits into independent chains: rows x and x+1 are linked when either is a
// lateral cell.  Each chain is walked in order by one thread, chains in
// parallel; cells of different chains never read or write each other, so the
// result is the serial loop's.  Cells linked to neither neighbour (most of
// them) only gather, all in parallel.
//
// A walker keeps the rows it works on - the previous, current and next row
// of its chain - in registers (ApplyRow) and touches memory once per row:
// all loads of the next row are issued together at the top of a step, and a
// row is written back when it leaves the window.  The grain store helpers
// below are sort_active :3874-3947 and slide_GS :4077-4171 on such rows.

// erodetot3 of every cell of the pass (0 where the cell is not processed)
__device__ __forceinline__ bool apply_active(const hc_view& c, size_t cell, int x) {
  return c.mask[cell] && dgt(c.h[cell], c.p.water_depth_erosion_threshold) && x < c.imax && x > 1;
}

// Per-cell terms of the apply pass that depend on the cell's own state and
// the (constant) outgoing fluxes only, computed for all cells in parallel:
// plane n (1..9) = incoming - outgoing bedload of fraction n, plane 0 =
// settled suspended load Vpdrop, plane 10 = erodetot.  The new Vsusptot is
// written directly (nothing else in the pass touches it).
__device__ __forceinline__ double& PRE(const hc_view& c, int k, size_t cell) {
  return c.pre[cell * kGrainStride + k];  // a cell's 11 terms side by side, like its record
}

__global__ void __launch_bounds__(256) k_apply_pre(const hc_view c, hc_dev* d) {
  if (!(d->it_active && d->rest_active && d->do_erode) || d->erode_retry) return;
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    d->xchains = 0;  // the chain lists are rebuilt by k_apply_gather
    d->ychains = 0;
    d->xresume = 0;
    d->yresume = 0;
    d->xtake = 0;
    d->ytake = 0;
  }
  if (y > c.jmax - 1 || x > c.imax) return;
  const size_t cell = (size_t)x * c.W + y;
  const size_t W = c.W;
  double et3 = 0;
  if (apply_active(c, cell, x)) {
    const hc_params& p = c.p;
    const double ts = d->s.time_step;
    const bool susp1 = p.isSuspended[1];
    // every flux is loaded before the first store: the stores would keep the
    // compiler from issuing a later fraction's loads ahead of them
    double val1[HC_G], val2[HC_G];
#pragma unroll
    for (int n = 1; n <= HC_G - 1; n++) {
      if (n == 1 && susp1) continue;
      val1[n] = (SF(c, 0, n, cell) + SF(c, 1, n, cell) + SF(c, 2, n, cell) + SF(c, 3, n, cell));
      val2[n] = (SF(c, 0, n, cell + 1) + SF(c, 2, n, cell - 1) + SF(c, 3, n, cell + W) +
                 SF(c, 1, n, cell - W));
    }
    double erodetot = 0, Vpdrop = 0, vs = 0;
    double dn[HC_G];
#pragma unroll
    for (int n = 1; n <= HC_G - 1; n++) {
      if (n == 1 && susp1) {
        const double ssv = c.ss[cell];
        vs = c.vs[cell] + ssv;
        erodetot -= ssv;
        // inputpointsarray is all false in the reference (zero_values clears
        // it after the reach block), so settling applies everywhere
        double coeff = ddiv_rn(p.fallVelocity[n] * ts, c.h[cell]);
        if (dgt(coeff, 1.0)) coeff = 1;
        Vpdrop = coeff * vs;
        if (dgt(Vpdrop, 0.001)) Vpdrop = 0.001;
        erodetot += Vpdrop;
        vs -= Vpdrop;
      } else {
        dn[n] = val2[n] - val1[n];
        erodetot += dn[n];
        et3 += val1[n];
      }
    }
    if (susp1) {
      c.vs[cell] = vs;
      PRE(c, 0, cell) = Vpdrop;
    }
#pragma unroll
    for (int n = 1; n <= HC_G - 1; n++)
      if (!(n == 1 && susp1)) PRE(c, n, cell) = dn[n];
    PRE(c, 10, cell) = erodetot;
  }
  c.erodetot3[cell] = et3;
}

// One lateral step of the apply passes (:4630-4677, :4690-4744) from a cell
// at elevation e0 (tau0, erodetot3 et3) toward its neighbour N.  Returns
// false when the raw amount is not positive; otherwise the (possibly zeroed
// or capped) amount, which the caller applies and hands to slide_GS even
// when it is zero, as the reference does.
__device__ __forceinline__ bool lateral_amount(const hc_params& p, const hc_divisor& dxd,
                                               double mult,
                                               double ts, double tau0, double et3,
                                               const ApplyRow& N, double e0, bool boundary,
                                               double& amt) {
  const double e_nb = N.elev;
  amt = 0;
  if (dlt(N.h, p.water_depth_erosion_threshold))
    amt = ddiv_by(mult * p.lateral_constant * tau0 * N.edge * ts, dxd);
  else
    amt = ddiv_by(p.chann_lateral_erosion * et3 * (e_nb - e0), dxd) * 0.1;
  if (!dgt0(amt)) return false;
  // amt *= 1 - veg * (1 - veg_lat_restriction): veg is zero (no vegetation)
  if (dlt(e_nb - amt, N.bed) || boundary) amt = 0;
  if (dgt(amt, p.ERODEFACTOR * 0.1)) amt = p.ERODEFACTOR * 0.1;
  return true;
}

// the lateral step of cell C (elevation e0) toward neighbour N
__device__ __forceinline__ void lateral_step(const hc_view& c, hc_dev* d, double mult, double ts,
                                             double tau0, double et3, size_t ccell, ApplyRow& C,
                                             double e0, size_t ncell, ApplyRow& N, bool boundary,
                                             double& elev_update, double totN) {
  const double en = N.elev;
  double amt;
  if (dgt(en, e0) && lateral_amount(c.p, c.dxd, mult, ts, tau0, et3, N, e0, boundary, amt)) {
    elev_update += amt;
    N.elev = en - amt;
    N.dirty = true;
    slide_GS_rows(c, d, ncell, N, amt, ccell, C, totN);
  }
}

// The lateral steps of C toward U, then toward D, through one copy of the
// step's code (the side's row goes through N): the walkers are bound by
// latency and instruction fetch, not by registers moves.
__device__ __forceinline__ void lateral_both(const hc_view& c, hc_dev* d, double mult, double ts,
                                             double tau0, double et3, size_t ccell, ApplyRow& C,
                                             double e0, bool doU, size_t ucell, ApplyRow& U,
                                             bool bU, bool doD, size_t dcell, ApplyRow& D,
                                             bool bD, double& elev_update) {
  // both rows' slide_GS totals, formed ahead and side by side (the slide
  // toward C changes neither U's nor D's fractions before its own slide)
  const double totU = doU ? positive_total(U) : 0.0;
  const double totD = doD ? positive_total(D) : 0.0;
#pragma unroll 1
  for (int side = 0; side < 2; side++) {
    if (!(side == 0 ? doU : doD)) continue;
    ApplyRow N = (side == 0) ? U : D;
    lateral_step(c, d, mult, ts, tau0, et3, ccell, C, e0, side == 0 ? ucell : dcell, N,
                 side == 0 ? bU : bD, elev_update, side == 0 ? totU : totD);
    if (side == 0) U = N;
    else D = N;
  }
}

// the gather of an active cell (:4579-4628): grain += incoming - outgoing,
// elev += erodetot, sort_active when the cell lost material.  Returns the
// new elevation.
__device__ __forceinline__ double gather_row(const hc_view& c, hc_dev* d, size_t cell,
                                             ApplyRow& r, const double* pre, double ss) {
  const bool susp1 = c.p.isSuspended[1] != 0;
#pragma unroll
  for (int n = 1; n <= HC_G - 1; n++) {
    if (n == 1 && susp1) {
      const double g = r.g[1] - ss;
      r.g[1] = g + pre[0];
    } else {
      r.g[n] += pre[n];
    }
  }
  const double erodetot = pre[10];
  const double e0 = r.elev + erodetot;
  r.elev = e0;
  r.dirty = true;
  if (dlt0(erodetot)) sort_active_row(c, d, cell, r);
  return e0;
}

__device__ __forceinline__ void load_pre(const hc_view& c, size_t cell, double* pre,
                                         double& ss) {
#pragma unroll
  for (int k = 0; k <= HC_G; k++) pre[k] = PRE(c, k, cell);
  ss = c.ss[cell];
}

// Isolated cells gather here, in parallel; chain starts of both passes go to
// the lists.  x pass: lat(r) = erodetot3 > 0 (r in 1..imax); a chain starts
// at x when rows x-1, x are not linked (or x == 1) and x is linked to x+1.
// y pass: lat(q) = wet-listed with erodetot3 > 0 (q in 2..jmax-1, rows
// 2..imax-1).
__global__ void __launch_bounds__(256) k_apply_gather(const hc_view c, hc_dev* d) {
  if (!(d->it_active && d->rest_active && d->do_erode) || d->erode_retry) return;
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > c.jmax - 1 || x > c.imax) return;
  const size_t W = c.W;
  const size_t cell = (size_t)x * W + y;
  const double* et3 = c.erodetot3;
  const bool lat0 = dgt0(et3[cell]);
  const bool latm = x - 1 >= 1 && dgt0(et3[cell - W]);
  const bool latp = x + 1 <= c.imax && dgt0(et3[cell + W]);
  const bool link_prev = latm || lat0, link_next = lat0 || latp;
  if (!(link_prev && x > 1)) {
    if (link_next) {
      const unsigned k = atomicAdd(&d->xchains, 1u);
      c.chains[k] = (uint32_t)cell;
    } else if (apply_active(c, cell, x)) {
      ApplyRow r;
      row_load(c, cell, EX(c, x, y), r);
      double pre[HC_G + 1], ss;
      load_pre(c, cell, pre, ss);
      gather_row(c, d, cell, r, pre, ss);
      row_store(c, cell, r);
    }
  }
  if (x >= 2 && x <= c.imax - 1) {
    auto lat = [&](int q) {
      return q >= 2 && q <= c.jmax - 1 && c.mask[cell - y + q] && dgt0(et3[cell - y + q]);
    };
    const bool l0 = lat(y);
    if (!((lat(y - 1) || l0) && y > 2) && (l0 || lat(y + 1))) {
      const unsigned k = atomicAdd(&d->ychains, 1u);
      c.chains[c.N2 + k] = (uint32_t)cell;
    }
  }
}

// Chains are walked by one thread each when there are many (all of them in
// flight at once), by one warp each when there are few (each one faster).
// With many, a thread walks the first kHandOff rows of its chain and hands a
// longer chain to the warp walkers: the rows it holds go back to memory and
// the rest of the chain is listed as a resume point (bit 31: the row before
// it is part of the chain).
// Blocks of 128 threads of the chain walkers, sized like entrain_blocks; a
// pass with no more chains than the launch has warps leaves them all to the
// warp walkers (both launches have the same grid, so both kernels see the
// same limit: gridDim.x * 4).
static unsigned walk_blocks(size_t N2) {
  return (unsigned)std::min<size_t>(152 * 8, std::max<size_t>(16, N2 / 2048));
}
__device__ __forceinline__ unsigned warps_in_flight() { return gridDim.x * (blockDim.x >> 5); }
constexpr int kHandOff = 32;
constexpr uint32_t kResumeU = 0x80000000u;

// A row's inputs to the walkers, staged in shared memory by asynchronous
// copies (cp.async): a walker asks for row r+2 before it works on row r, so
// the copies' latency hides behind that work.  One slot per thread.
struct StagedRow {
  double g[HC_G + 1];
  double pre[HC_G + 1];
  double elev, h, bed, edge, tau, ss, et3;
  int idx;
  unsigned int mword;  // the aligned 4-byte word that holds mask[cell]
};

__device__ __forceinline__ void cp_async(void* smem, const void* gmem, int bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if (bytes == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__device__ __forceinline__ void stage_issue(const hc_view& c, StagedRow* st, size_t cell,
                                            size_t ecell, bool with_pre) {
  for (int n = 0; n <= HC_G; n++) cp_async(&st->g[n], &GRN(c, cell, n), 8);
  if (with_pre)
    for (int k = 0; k <= HC_G; k++) cp_async(&st->pre[k], &PRE(c, k, cell), 8);
  cp_async(&st->elev, c.elev + cell, 8);
  cp_async(&st->h, c.h + cell, 8);
  cp_async(&st->bed, c.bed + cell, 8);
  cp_async(&st->edge, c.edge + ecell, 8);
  cp_async(&st->tau, c.tau + cell, 8);
  cp_async(&st->ss, c.ss + cell, 8);
  cp_async(&st->et3, c.erodetot3 + cell, 8);
  cp_async(&st->idx, c.index + cell, 4);
  cp_async(&st->mword, (const void*)((uintptr_t)(c.mask + cell) & ~(uintptr_t)3), 4);
  cp_async_commit();
}

// waits for the slot and moves it into registers
__device__ __forceinline__ void stage_take(const StagedRow* st, size_t cell, ApplyRow& r,
                                           double* pre, double& tau, double& ss, double& et3,
                                           bool& mask) {
  cp_async_wait_all();
#pragma unroll
  for (int n = 0; n <= HC_G; n++) r.g[n] = st->g[n];
  if (pre)
#pragma unroll
    for (int k = 0; k <= HC_G; k++) pre[k] = st->pre[k];
  r.elev = st->elev;
  r.h = st->h;
  r.bed = st->bed;
  r.edge = st->edge;
  r.idx = st->idx;
  r.dirty = false;
  tau = st->tau;
  ss = st->ss;
  et3 = st->et3;
  mask = ((st->mword >> (8 * (unsigned)(cell & 3))) & 0xffu) != 0;
}

// The next chain for the lanes of a warp that need one (one atomic per
// warp): the chains are taken in list order as lanes free up, so a lane
// whose chain ended does not wait for the longest chain of its warp.
// Returns the chain number (>= nch: none left).
__device__ __forceinline__ unsigned take_chain(unsigned* counter, bool need) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned b = __ballot_sync(0xffffffffu, need);
  if (!b) return ~0u;
  const unsigned leader = __ffs(b) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(b));
  base = __shfl_sync(0xffffffffu, base, leader);
  return base + __popc(b & ((1u << lane) - 1));
}

// chains along the columns, one per thread (many chains): rows r-1, r, r+1
// held in U, C, D; one row per turn of the loop, a new chain as soon as the
// lane's chain ends
__global__ void __launch_bounds__(128) k_apply_xchains_t(const hc_view c, hc_dev* d) {
  __shared__ StagedRow slots[128];
  if (!(d->it_active && d->rest_active && d->do_erode) || d->erode_retry) return;
  if (d->xchains <= warps_in_flight()) return;  // few chains: the warp walker takes them
  StagedRow* st = &slots[threadIdx.x];
  const unsigned nch = d->xchains;
  const double mult = d->mult, ts = d->s.time_step;
  const double thr = c.p.water_depth_erosion_threshold;
  const size_t W = c.W;
  auto active = [&](bool m, double h, int x) { return m && dgt(h, thr) && x < c.imax && x > 1; };
  ApplyRow U, C, D;
  double Cpre[HC_G + 1], Dpre[HC_G + 1];
  double Ctau = 0, Css = 0, Cet3 = 0;
  bool Cm, Dm, Cact = false, hasU = false;
  size_t cell = 0, ucell = 0;
  int y = 0, r = 0, steps = 0;
  bool live = false, done = false;
  for (;;) {
    const unsigned k = take_chain(&d->xtake, !live && !done);
    if (!live && !done) {
      if (k < nch) {
        cell = c.chains[k];
        y = (int)(cell % W);
        r = (int)(cell / W);
        stage_issue(c, st, cell, EX(c, r, y), true);
        stage_take(st, cell, C, Cpre, Ctau, Css, Cet3, Cm);
        Cact = active(Cm, C.h, r);
        if (r + 1 <= c.imax) stage_issue(c, st, cell + W, EX(c, r + 1, y), true);
        steps = 0;
        hasU = false;
        live = true;
      } else {
        done = true;
      }
    }
    if (!__any_sync(0xffffffffu, live)) break;
    if (!live) continue;
    const bool hasD = r + 1 <= c.imax;
    const size_t dcell = cell + W;
    double Det3 = 0, Dtau = 0, Dss = 0;
    bool Dact = false;
    if (hasD) {
      stage_take(st, dcell, D, Dpre, Dtau, Dss, Det3, Dm);
      Dact = active(Dm, D.h, r + 1);
      // row r+2 is copied while row r is worked on
      if (r + 2 <= c.imax) stage_issue(c, st, dcell + W, EX(c, r + 2, y), true);
    }
    if (Cact) {
      const double e0 = gather_row(c, d, cell, C, Cpre, Css);
      if (dgt0(Cet3)) {
        double elev_update = 0;
        lateral_both(c, d, mult, ts, Ctau, Cet3, cell, C, e0, r > 2 && hasU, ucell, U,
                     r - 1 == 1, r < c.imax - 1 && hasD, dcell, D, r + 1 == c.imax,
                     elev_update);
        C.elev = C.elev + elev_update;
      }
    }
    if (hasU) row_store(c, ucell, U);  // row r-1 is final
    if (!(dgt0(Cet3) || dgt0(Det3)) || !hasD) {
      row_store(c, cell, C);
      if (hasD) row_store(c, dcell, D);
      cp_async_wait_all();  // the slot is free for the next chain
      live = false;
      continue;
    }
    if (++steps >= kHandOff) {  // a long chain: the warp walkers go on from row r+1
      row_store(c, cell, C);
      row_store(c, dcell, D);
      cp_async_wait_all();
      const unsigned m = atomicAdd(&d->xresume, 1u);
      c.chains[2 * c.N2 + m] = (uint32_t)dcell | kResumeU;
      live = false;
      continue;
    }
    U = C;
    hasU = true;
    ucell = cell;
    C = D;
#pragma unroll
    for (int n = 0; n <= HC_G; n++) Cpre[n] = Dpre[n];
    Ctau = Dtau;
    Css = Dss;
    Cet3 = Det3;
    Cact = Dact;
    cell = dcell;
    r++;
  }
}

// chains along the rows for the +/-y pass: columns q-1, q, q+1 held in
// U, C, D; one column per turn of the loop, a new chain as soon as the
// lane's chain ends
__global__ void __launch_bounds__(128) k_apply_ychains_t(const hc_view c, hc_dev* d) {
  __shared__ StagedRow slots[128];
  if (!(d->it_active && d->rest_active && d->do_erode) || d->erode_retry) return;
  if (d->ychains <= warps_in_flight()) return;
  StagedRow* st = &slots[threadIdx.x];
  const unsigned nch = d->ychains;
  const double mult = d->mult, ts = d->s.time_step;
  const size_t W = c.W;
  auto lat = [&](int qq, bool m, double et3) { return qq >= 2 && qq <= c.jmax - 1 && m && dgt0(et3); };
  ApplyRow U, C, D;
  double Ctau = 0, Css = 0, Cet3 = 0, t0, t1, t2;
  bool Cm, Dm, m0, Clat = false;
  size_t cell = 0;
  int x = 0, q = 0, steps = 0;
  bool live = false, done = false;
  for (;;) {
    const unsigned k = take_chain(&d->ytake, !live && !done);
    if (!live && !done) {
      if (k < nch) {
        cell = c.chains[c.N2 + k];
        x = (int)(cell / W);
        q = (int)(cell % W);
        stage_issue(c, st, cell - 1, EX(c, x, q - 1), false);
        stage_take(st, cell - 1, U, nullptr, t0, t1, t2, m0);
        stage_issue(c, st, cell, EX(c, x, q), false);
        stage_take(st, cell, C, nullptr, Ctau, Css, Cet3, Cm);
        Clat = lat(q, Cm, Cet3);
        stage_issue(c, st, cell + 1, EX(c, x, q + 1), false);  // q + 1 <= jmax
        steps = 0;
        live = true;
      } else {
        done = true;
      }
    }
    if (!__any_sync(0xffffffffu, live)) break;
    if (!live) continue;
    const size_t dcell = cell + 1;
    double Dtau, Dss, Det3;
    stage_take(st, dcell, D, nullptr, Dtau, Dss, Det3, Dm);
    const bool Dlat = lat(q + 1, Dm, Det3);
    if (q + 2 <= c.jmax) stage_issue(c, st, dcell + 1, EX(c, x, q + 2), false);
    if (Clat) {
      const double e0 = C.elev;
      double elev_update = 0;
      lateral_both(c, d, mult, ts, Ctau, Cet3, cell, C, e0, true, cell - 1, U, q - 1 == 1, true,
                   dcell, D, q + 1 == c.jmax, elev_update);
      C.elev = C.elev + elev_update;
      C.dirty = true;
    }
    row_store(c, cell - 1, U);  // column q-1 is final
    if (!(Clat || Dlat) || q + 1 > c.jmax - 1) {
      row_store(c, cell, C);
      row_store(c, dcell, D);
      cp_async_wait_all();
      live = false;
      continue;
    }
    if (++steps >= kHandOff) {  // a long chain: the warp walkers go on from column q+1
      row_store(c, cell, C);
      row_store(c, dcell, D);
      cp_async_wait_all();
      const unsigned m = atomicAdd(&d->yresume, 1u);
      c.chains[3 * c.N2 + m] = (uint32_t)dcell;
      live = false;
      continue;
    }
    U = C;
    C = D;
    Ctau = Dtau;
    Css = Dss;
    Cet3 = Det3;
    Clat = Dlat;
    cell = dcell;
    q++;
  }
}

// ---------------------------------------------------------------------------
// The chain walkers.  One warp per chain: lane n holds fraction n of each
// held row's grain record (lanes 0..HC_G), so the per-fraction arithmetic of
// the gather, slide_GS and sort_active runs as one instruction for all
// fractions instead of nine; the FP64 pipe, a few lanes per clock on this
// GPU, is what a single walker waits on.  Sums keep the reference's order
// (sequential over the fractions, every lane forming the same sum), so the
// results are the serial loop's.  Rows r-1, r, r+1 are held (U, C, D) and
// row r+2 is loaded while row r is worked on.
// ---------------------------------------------------------------------------
constexpr unsigned kFull = 0xffffffffu;

struct WRow {
  double g;  // grain plane `lane` (lanes 0..HC_G; 0 in the others)
  double elev, h, bed, edge;
  int idx;
  bool dirty;
};

// the rest of a row the x walker needs when it is the current row
struct WExtra {
  double pre;  // PRE plane `lane` (lanes 0..HC_G)
  double tau, ss, et3;
  bool mask;
};

__device__ __forceinline__ int lane_id() { return (int)(threadIdx.x & 31); }

__device__ __forceinline__ void wrow_load(const hc_view& c, size_t cell, size_t ecell, WRow& r) {
  const int L = lane_id();
  r.g = (L <= HC_G) ? GRN(c, cell, L) : 0.0;
  r.elev = c.elev[cell];
  r.h = c.h[cell];
  r.bed = c.bed[cell];
  r.edge = c.edge[ecell];
  r.idx = c.index[cell];
  r.dirty = false;
}

__device__ __forceinline__ void wextra_load(const hc_view& c, size_t cell, bool with_pre,
                                            WExtra& x) {
  const int L = lane_id();
  x.pre = (with_pre && L <= HC_G) ? PRE(c, L, cell) : 0.0;
  x.tau = c.tau[cell];
  x.ss = c.ss[cell];
  x.et3 = c.erodetot3[cell];
  x.mask = c.mask[cell] != 0;
}

__device__ __forceinline__ void wrow_store(const hc_view& c, size_t cell, const WRow& r) {
  if (!r.dirty) return;
  const int L = lane_id();
  if (L >= 1 && L <= HC_G - 1) GRN(c, cell, L) = r.g;
  if (L == 0) c.elev[cell] = r.elev;
}

// sort_active on a held row, the warp together (same decisions as
// sort_active_row; the float estimate's sum order does not matter, its
// error bound holds for any order)
__device__ void sort_active_w(const hc_view& c, hc_dev* d, size_t cell, WRow& r) {
  const int L = lane_id();
  if (r.idx == -9999) {
    if (L == 0) {
      d->err_code = 201;
      d->pause |= HC_PAUSE_ERROR;
    }
    return;
  }
  const double active = c.p.active;
  const float f = (L <= HC_G) ? approx_f(r.g) : 0.0f;
  float sf = f, af = fabsf(f);
  for (int o = 16; o > 0; o >>= 1) {
    sf += __shfl_xor_sync(kFull, sf, o);
    af += __shfl_xor_sync(kFull, af, o);
  }
  const float tol = 1e-5f * af + 1e-30f;
  const float hi = c.act_hi, lo = c.act_lo;
  const int dep = (sf > hi + tol) ? 1 : ((sf < hi - tol) ? -1 : 0);
  const int ero = (sf < lo - tol) ? 1 : ((sf > lo + tol) ? -1 : 0);
  if (dep == -1 && ero == -1) return;
  double total = 0.0;  // in the reference's order, n = 0 .. HC_G
  for (int n = 0; n <= HC_G; n++) total += __shfl_sync(kFull, r.g, n);
  if (total > (active * 1.5)) {
    if (L <= HC_G - 2)
      for (int z = 9; z >= 1; z--) STR(c, cell, z, L) = STR(c, cell, z - 1, L);
    __syncwarp();
    const double coeff = active / total;
    if (L >= 1 && L <= HC_G - 1 && r.g > 0.0) {
      const double amount = coeff * (r.g);
      STR(c, cell, 0, L - 1) = amount;
      r.g = r.g - amount;
    }
    r.dirty = true;
    __syncwarp();
  }
  if (total < (active / 4)) {
    double s0 = 0;
    if (L >= 1 && L <= HC_G - 1) s0 = STR(c, cell, 0, L - 1);
    __syncwarp();
    if (L <= HC_G - 2)
      for (int z = 0; z <= 8; z++) STR(c, cell, z, L) = STR(c, cell, z + 1, L);
    __syncwarp();
    if (L >= 1 && L <= HC_G - 1) {
      r.g += s0;
      STR(c, cell, 9, L - 1) = active * c.p.dprop[L];
    }
    r.dirty = true;
    __syncwarp();
  }
}

// slide_GS(a -> b, amount) on held rows, the warp together
__device__ void slide_GS_w(const hc_view& c, hc_dev* d, size_t a, WRow& A, double amount,
                           size_t b, WRow& B) {
  const int L = lane_id();
  const bool fr = L >= 1 && L <= HC_G - 1;
  const double dp = fr ? c.p.dprop[L] : 0.0;
  const bool ha = A.idx != -9999, hb = B.idx != -9999;
  if (ha && hb) {
    double total = 0;  // positive fractions 1..9, in order
    for (int n = 1; n <= HC_G - 1; n++) {
      const double v = __shfl_sync(kFull, A.g, n);
      if (dgt0(v)) total += v;
    }
    if (dgt(amount, total)) {
      if (fr) B.g += (amount - total) * dp;
      amount = total;
    }
    if (dgt0(total)) {
      if (fr) {
        const double ga = A.g;
        const double t = amount * ddiv_rn(ga, total);
        B.g += t;
        double na = ga - t;
        if (dlt0(na)) na = 0;
        A.g = na;
      }
    }
    A.dirty = B.dirty = true;
    sort_active_w(c, d, a, A);
    sort_active_w(c, d, b, B);
    return;
  }
  if (!ha && hb) {
    if (fr) B.g += (amount)*dp;
    B.dirty = true;
    sort_active_w(c, d, b, B);
    return;
  }
  if (ha && !hb && L == 0) {
    d->err_code = 202;
    d->pause |= HC_PAUSE_ERROR;
  }
}

__device__ __forceinline__ bool lateral_amount_w(const hc_params& p, const hc_divisor& dxd,
                                                 double mult,
                                                 double ts, double tau0, double et3,
                                                 const WRow& N, double e0, bool boundary,
                                                 double& amt) {
  const double e_nb = N.elev;
  amt = 0;
  if (dlt(N.h, p.water_depth_erosion_threshold))
    amt = ddiv_by(mult * p.lateral_constant * tau0 * N.edge * ts, dxd);
  else
    amt = ddiv_by(p.chann_lateral_erosion * et3 * (e_nb - e0), dxd) * 0.1;
  if (!dgt0(amt)) return false;
  if (dlt(e_nb - amt, N.bed) || boundary) amt = 0;
  if (dgt(amt, p.ERODEFACTOR * 0.1)) amt = p.ERODEFACTOR * 0.1;
  return true;
}

__device__ __forceinline__ void lateral_step_w(const hc_view& c, hc_dev* d, double mult,
                                               double ts, double tau0, double et3, size_t ccell,
                                               WRow& C, double e0, size_t ncell, WRow& N,
                                               bool boundary, double& elev_update) {
  const double en = N.elev;
  double amt;
  if (dgt(en, e0) && lateral_amount_w(c.p, c.dxd, mult, ts, tau0, et3, N, e0, boundary, amt)) {
    elev_update += amt;
    N.elev = en - amt;
    N.dirty = true;
    slide_GS_w(c, d, ncell, N, amt, ccell, C);
  }
}

// the gather of an active cell, the warp together
__device__ __forceinline__ double gather_w(const hc_view& c, hc_dev* d, size_t cell, WRow& r,
                                           const WExtra& x) {
  const int L = lane_id();
  const double pre0 = __shfl_sync(kFull, x.pre, 0);
  const double erodetot = __shfl_sync(kFull, x.pre, HC_G);
  if (L >= 1 && L <= HC_G - 1) {
    if (L == 1 && c.p.isSuspended[1]) {
      const double g = r.g - x.ss;
      r.g = g + pre0;
    } else {
      r.g += x.pre;
    }
  }
  const double e0 = r.elev + erodetot;
  r.elev = e0;
  r.dirty = true;
  if (dlt0(erodetot)) sort_active_w(c, d, cell, r);
  return e0;
}

// chains along the columns, one warp per chain
__global__ void __launch_bounds__(128) k_apply_xchains_w(const hc_view c, hc_dev* d) {
  if (!(d->it_active && d->rest_active && d->do_erode) || d->erode_retry) return;
  // few chains: all of them from their starts; many: the long ones the
  // thread walker handed over
  const bool few = d->xchains <= warps_in_flight();
  const unsigned nch = few ? d->xchains : d->xresume;
  const uint32_t* list = c.chains + (few ? 0 : 2 * c.N2);
  const double mult = d->mult, ts = d->s.time_step;
  const double thr = c.p.water_depth_erosion_threshold;
  const size_t W = c.W;
  const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
  auto active = [&](const WExtra& x, double h, int r) {
    return x.mask && h > thr && r < c.imax && r > 1;
  };
  for (unsigned k = warp; k < nch; k += nwarps) {
    const uint32_t rec = list[k];
    size_t cell = rec & ~kResumeU;
    const int y = (int)(cell % W);
    int r = (int)(cell / W);
    WRow U, C, D, E;
    WExtra Cx, Dx, Ex;
    bool hasU = (rec & kResumeU) != 0;
    size_t ucell = cell - W;
    if (hasU) wrow_load(c, ucell, EX(c, r - 1, y), U);
    wrow_load(c, cell, EX(c, r, y), C);
    wextra_load(c, cell, true, Cx);
    if (r + 1 <= c.imax) {
      wrow_load(c, cell + W, EX(c, r + 1, y), D);
      wextra_load(c, cell + W, true, Dx);
    }
    bool Cact = active(Cx, C.h, r);
    for (;;) {
      const bool hasD = r + 1 <= c.imax;
      const size_t dcell = cell + W;
      // row r+2, loaded while row r is worked on
      const bool hasE = r + 2 <= c.imax;
      if (hasE) {
        wrow_load(c, dcell + W, EX(c, r + 2, y), E);
        wextra_load(c, dcell + W, true, Ex);
      }
      const double Det3 = hasD ? Dx.et3 : 0.0;
      const bool Dact = hasD && active(Dx, D.h, r + 1);
      if (Cact) {
        const double e0 = gather_w(c, d, cell, C, Cx);
        if (Cx.et3 > 0) {
          double elev_update = 0;
          if (r > 2 && hasU)
            lateral_step_w(c, d, mult, ts, Cx.tau, Cx.et3, cell, C, e0, ucell, U, r - 1 == 1,
                           elev_update);
          if (r < c.imax - 1 && hasD)
            lateral_step_w(c, d, mult, ts, Cx.tau, Cx.et3, cell, C, e0, dcell, D,
                           r + 1 == c.imax, elev_update);
          C.elev = C.elev + elev_update;
        }
      }
      if (hasU) wrow_store(c, ucell, U);  // row r-1 is final
      if (!(Cx.et3 > 0 || Det3 > 0) || !hasD) {
        wrow_store(c, cell, C);
        if (hasD) wrow_store(c, dcell, D);
        break;
      }
      U = C;
      hasU = true;
      ucell = cell;
      C = D;
      Cx = Dx;
      Cact = Dact;
      D = E;
      Dx = Ex;
      cell = dcell;
      r++;
    }
  }
}

// chains along the rows for the +/-y pass, one warp per chain: columns
// q-1, q, q+1 held in U, C, D
__global__ void __launch_bounds__(128) k_apply_ychains_w(const hc_view c, hc_dev* d) {
  if (!(d->it_active && d->rest_active && d->do_erode) || d->erode_retry) return;
  const bool few = d->ychains <= warps_in_flight();
  const unsigned nch = few ? d->ychains : d->yresume;
  const uint32_t* list = c.chains + (few ? 1 : 3) * c.N2;
  const double mult = d->mult, ts = d->s.time_step;
  const size_t W = c.W;
  const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
  for (unsigned k = warp; k < nch; k += nwarps) {
    size_t cell = list[k];
    const int x = (int)(cell / W);
    int q = (int)(cell % W);
    auto lat = [&](int qq, const WExtra& e) {
      return qq >= 2 && qq <= c.jmax - 1 && e.mask && e.et3 > 0;
    };
    WRow U, C, D, E;
    WExtra Cx, Dx, Ex;
    wrow_load(c, cell - 1, EX(c, x, q - 1), U);
    wrow_load(c, cell, EX(c, x, q), C);
    wextra_load(c, cell, false, Cx);
    wrow_load(c, cell + 1, EX(c, x, q + 1), D);  // q + 1 <= jmax
    wextra_load(c, cell + 1, false, Dx);
    bool Clat = lat(q, Cx);
    for (;;) {
      const size_t dcell = cell + 1;
      const bool hasE = q + 2 <= c.jmax;
      if (hasE) {
        wrow_load(c, dcell + 1, EX(c, x, q + 2), E);
        wextra_load(c, dcell + 1, false, Ex);
      }
      const bool Dlat = lat(q + 1, Dx);
      if (Clat) {
        const double e0 = C.elev;
        double elev_update = 0;
        lateral_step_w(c, d, mult, ts, Cx.tau, Cx.et3, cell, C, e0, cell - 1, U, q - 1 == 1,
                       elev_update);
        lateral_step_w(c, d, mult, ts, Cx.tau, Cx.et3, cell, C, e0, dcell, D, q + 1 == c.jmax,
                       elev_update);
        C.elev = C.elev + elev_update;
        C.dirty = true;
      }
      wrow_store(c, cell - 1, U);  // column q-1 is final
      if (!(Clat || Dlat) || q + 1 > c.jmax - 1) {
        wrow_store(c, cell, C);
        wrow_store(c, dcell, D);
        break;
      }
      U = C;
      C = D;
      Cx = Dx;
      Clat = Dlat;
      D = E;
      Dx = Ex;
      cell = dcell;
      q++;
    }
  }
}

// ---------------------------------------------------------------------------
// sediment leaving the edges :4750-4841.  The reference accumulates gtot2 in
// float, entry by entry in its loop order: the contributions are laid out in
// that order, one plane per fraction, and each fraction's float sum is run in
// order by its own warp.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_edge_out(const hc_view c, hc_dev* d, double* contrib,
                                                    int32_t* list, int post) {
  __shared__ int cnt_s[1024];
  __shared__ float gsum[HC_G + 1];
  if (!(d->it_active && d->rest_active && d->do_erode) || d->erode_retry) return;
  const hc_params& p = c.p;
  const int imax = c.imax, jmax = c.jmax;
  const double thr = p.water_depth_erosion_threshold;
  const int nA = (jmax - 2 > 0) ? 2 * (jmax - 2) : 0;   // y = 2..jmax-1: (imax,y), (1,y)
  const int nB = (imax - 2 > 0) ? 2 * (imax - 2) : 0;   // x = 2..imax-1: (x,jmax), (x,1)
  const int ntot = nA + nB;
  const size_t cap = (size_t)(2 * (imax + jmax) + 8);  // entries per fraction plane
  // entries handled by this thread: a contiguous chunk, so the block scan
  // below keeps the loop order
  const int per = (ntot + blockDim.x - 1) / blockDim.x;
  const int k0 = threadIdx.x * per, k1 = min(ntot, k0 + per);
  int mine = 0;
  for (int k = k0; k < k1; k++) {
    int x, y;  // the sources: sr[imax-1][y], sl[2][y], sd[x][jmax-1], su[x][2]
    if (k < nA) {
      y = 2 + k / 2;
      x = ((k & 1) == 0) ? imax : 1;
    } else {
      const int kk = k - nA;
      x = 2 + kk / 2;
      y = ((kk & 1) == 0) ? jmax : 1;
    }
    const size_t cell = (size_t)x * c.W + y;
    if (c.h[cell] > thr || c.vs[cell] > 0) mine++;
  }
  cnt_s[threadIdx.x] = mine;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int t = 0; t < (int)blockDim.x; t++) {
      int v = cnt_s[t];
      cnt_s[t] = s;
      s += v;
    }
    d->misc_done = s;
  }
  __syncthreads();
  int o = cnt_s[threadIdx.x];
  for (int k = k0; k < k1; k++) {
    int x, y, srcx, srcy, dir;
    if (k < nA) {
      y = 2 + k / 2;
      if ((k & 1) == 0) { x = imax; srcx = imax - 1; srcy = y; dir = 1; }
      else { x = 1; srcx = 2; srcy = y; dir = 3; }
    } else {
      const int kk = k - nA;
      x = 2 + kk / 2;
      if ((kk & 1) == 0) { y = jmax; srcx = x; srcy = jmax - 1; dir = 2; }
      else { y = 1; srcx = x; srcy = 2; dir = 0; }
    }
    const size_t cell = (size_t)x * c.W + y;
    if (!(c.h[cell] > thr || c.vs[cell] > 0)) continue;
    const size_t src = (size_t)srcx * c.W + srcy;
    bool first_susp = true;  // Vsusptot is zeroed after the first suspended fraction
    for (int n = 1; n <= HC_G - 1; n++) {
      double v;
      if (p.isSuspended[n]) {
        v = first_susp ? c.vs[cell] : 0.0;
        first_susp = false;
      } else {
        v = SF(c, dir, n, src);
      }
      contrib[(size_t)n * cap + o] = v;
    }
    o++;
  }
  __syncthreads();
  // the suspended load leaves with the water (Vsusptot = 0 at these cells);
  // done after all reads above
  for (int k = k0; k < k1; k++) {
    int x, y;
    if (k < nA) {
      y = 2 + k / 2;
      x = ((k & 1) == 0) ? imax : 1;
    } else {
      const int kk = k - nA;
      x = 2 + kk / 2;
      y = ((kk & 1) == 0) ? jmax : 1;
    }
    const size_t cell = (size_t)x * c.W + y;
    if (c.h[cell] > thr || c.vs[cell] > 0) {
      bool anysusp = false;
      for (int n = 1; n <= HC_G - 1; n++) anysusp |= (p.isSuspended[n] != 0);
      if (anysusp) c.vs[cell] = 0;
    }
  }
  __syncthreads();
  const int total = d->misc_done;
  // fraction n's sum, by warp n: the warp loads 32 contributions at a time
  // and every lane adds them in order from registers
  const int wn = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (wn >= 1 && wn <= HC_G - 1) {
    const double* cn = contrib + (size_t)wn * cap;
    float g = 0.0f;
    // a zero contribution leaves g unchanged ((double)g + 0 == (double)g,
    // and g, starting at +0 with nothing to cancel to -0, is never -0), so
    // only the nonzero ones enter the chain of roundings
    for (int e0 = 0; e0 < total; e0 += 32) {
      const double v = (e0 + lane < total) ? cn[e0 + lane] : 0.0;
      unsigned nz = __ballot_sync(0xffffffffu, !deq0(v));
      while (nz) {
        const int k = __ffs(nz) - 1;
        nz &= nz - 1;
        g = d2f_i(f2d_i(g) + __shfl_sync(0xffffffffu, v, k));
      }
    }
    if (lane == 0) gsum[wn] = g;
  }
  if (threadIdx.x == 0) gsum[0] = 0.0f, gsum[HC_G] = 0.0f;
  __syncthreads();
  if (threadIdx.x == 0) {
    hc_scalars& s = d->s;
    const double DX = p.DX;
    s.sediQ = 0;
    for (int n = 1; n <= HC_G; n++) {
      s.sediQ += gsum[n] * DX * DX;
      s.globalsediq += gsum[n] * DX * DX;
      s.sum_grain[n] += gsum[n] * DX * DX;
    }
    // call_erosion :2277-2294 after erode() returned (post: the iteration's
    // own erosion call, not a measurement launch)
    if (post) {
      s.erode_mult = x86_trunc_to_int(p.ERODEFACTOR / s.tempbmax);
      if (s.erode_mult < 1) s.erode_mult = 1;
      if (s.erode_mult > 5) s.erode_mult = 5;
      s.erode_call = s.counter + s.erode_mult;
    }
  }
}

// call_lateral :2298-2305 (main.cpp:178, when enabled) is tested every
// iteration after call_erosion; lateral3 itself runs on the host-driven path
// before water_flux_out, so the rest of the iteration waits for it.
__global__ void k_lateral_check(const hc_view c, hc_dev* d) {
  if (!(d->it_active && d->rest_active)) return;
  if (c.p.hydro_only || !(d->flags & HC_RUN_LATERAL)) return;
  if (d->s.counter >= d->s.lateralcounter) {
    d->do_lateral = 1;
    d->rest_active = 0;
    d->pause |= HC_PAUSE_LATERAL;
  }
}

}  // namespace

// ------------------------------------------------------------------ launches
struct ErodeScratch {
  uint32_t* bits;      // N2/4+1 words
  int32_t* block_sums;
  int32_t* total;
  double* contrib;     // edge contributions
};

static ErodeScratch scratch_of(hc_ctx* c) {
  ErodeScratch s;
  char* base = (char*)c->v.red;
  s.total = (int32_t*)(base + 64);
  s.block_sums = (int32_t*)(base + 128);
  size_t nwords = c->v.N2 / 4 + 1;
  size_t nblocks = (nwords + 1023) / 1024;
  s.bits = (uint32_t*)(base + 128 + ((nblocks * 4 + 255) / 256) * 256);
  s.contrib = (double*)((char*)s.bits + ((nwords * 4 + 255) / 256) * 256);
  return s;
}

size_t erode_scratch_bytes(size_t N2, int imax, int jmax) {
  size_t nwords = N2 / 4 + 1;
  size_t nblocks = (nwords + 1023) / 1024;
  size_t ncontrib = (size_t)(2 * (imax + jmax) + 8) * HC_G;
  return 128 + ((nblocks * 4 + 255) / 256) * 256 + ((nwords * 4 + 255) / 256) * 256 +
         ncontrib * 8 + 256;
}

void launch_erode_begin(hc_ctx* c, int gated, double mult) {
  k_erode_begin<<<1, 1, 0, c->cs>>>(c->v, c->dev, gated, mult);
  count_launch(c, 1);
}

void launch_erode_pass(hc_ctx* c, int max_passes, cudaGraphConditionalHandle next, int has_next) {
  ErodeScratch s = scratch_of(c);
  dim3 b(32, 4);
  dim3 g((c->v.jmax - 1 + b.x - 1) / b.x, (c->v.imax + b.y - 1) / b.y);
  if (g.x < 1) g.x = 1;
  k_entrain_tau<<<g, b, 0, c->cs>>>(c->v, c->dev);
  k_entrain<<<entrain_blocks(c->v.N2), 128, 0, c->cs>>>(c->v, c->dev, max_passes, next,
                                                          has_next);
  count_launch(c, 2);
  size_t nwords = c->v.N2 / 4 + 1;
  int nb = (int)((c->v.N2 + 255) / 256);
  k_alloc_mark<<<nb, 256, 0, c->cs>>>(c->v, c->dev, s.bits);
  count_launch(c, 1);
  int nblocks = (int)((nwords + 1023) / 1024);
  k_alloc_count<<<nblocks, 1024, 0, c->cs>>>(c->v, c->dev, s.bits, s.block_sums, nwords,
                                             s.total);
  count_launch(c, 1);
  k_alloc_assign<<<nblocks, 1024, 0, c->cs>>>(c->v, c->dev, s.bits, s.block_sums, nwords,
                                              s.total);
  count_launch(c, 1);
}

void launch_erode_finish(hc_ctx* c, int gated) {
  ErodeScratch s = scratch_of(c);
  dim3 b(32, 8);
  dim3 g((c->v.jmax - 2 + 31) / 32, (c->v.imax + 7) / 8);
  k_apply_pre<<<g, b, 0, c->cs>>>(c->v, c->dev);
  k_apply_gather<<<g, b, 0, c->cs>>>(c->v, c->dev);
  const unsigned wb = walk_blocks(c->v.N2);
  k_apply_xchains_t<<<wb, 128, 0, c->cs>>>(c->v, c->dev);
  k_apply_xchains_w<<<wb, 128, 0, c->cs>>>(c->v, c->dev);
  k_apply_ychains_t<<<wb, 128, 0, c->cs>>>(c->v, c->dev);
  k_apply_ychains_w<<<wb, 128, 0, c->cs>>>(c->v, c->dev);
  count_launch(c, 6);
  k_edge_out<<<1, 1024, 0, c->cs>>>(c->v, c->dev, s.contrib, nullptr, gated);
  count_launch(c, 1);
}

void launch_lateral_check(hc_ctx* c) {
  k_lateral_check<<<1, 1, 0, c->cs>>>(c->v, c->dev);
  count_launch(c, 1);
}
