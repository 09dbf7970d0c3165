// lateral_channel_erode :4850-5291 ("lateral3"): the channel-edge curvature
// field `edge` that erode() uses for lateral bank erosion.
//
// The reference indexes its scratch arrays and `edge` with x < jmax+1 and
// y < imax+1, which only describes the grid for square domains; the library
// runs lateral3 on square grids and reports HC_ERR_UNSUPPORTED otherwise.
//
// Passes (all one thread per cell, Jacobi-style as in the reference):
//   L1  water_depth2 from Tau with isolated cells removed       :4863-4890
//   L2  edge cells and the 2x upscaled wet/dry grid              :4894-4939
//   L3  edge marks on the upscaled grid                          :4942-4958
//   L4  inside/outside tally on the upscaled grid                :4961-4991
//   L5  edge values from the tally                               :4994-5009
//   L6  edge_smoothing_passes + downstream_shift smoothing       :5011-5208
//   L7  curvature transform                                      :5210-5227
//   L8  cross-channel smoothing until converged                  :5229-5288
// In L6 and L8 a down_scan entry of row 1 or row jmax is processed at row 2
// or jmax-1 (the reference bumps x); those few entries of each column are
// handled by one thread per column so that their writes land in the
// reference's order.

#include "hc_grain.cuh"

#include <math.h>

namespace {

__constant__ int kLx[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1};
__constant__ int kLy[9] = {0, -1, -1, 0, 1, 1, 1, 0, -1};

constexpr double kMft = 0.1;

struct LatBufs {
  double* et;     // edge_temp  (jmax+1)(imax+1)
  double* wd2;    // water_depth2
  int* up;        // upscale (2(jmax+1)) x (2(imax+1))
  int* upe;       // upscale_edge
  double* diff;   // convergence measure
};

__device__ __forceinline__ size_t L(const hc_view& c, int x, int y) {
  return (size_t)x * (c.imax + 1) + y;
}
__device__ __forceinline__ size_t U(const hc_view& c, int x, int y) {
  return (size_t)x * (2 * (c.imax + 1)) + y;
}
__device__ __forceinline__ double& EDG(const hc_view& c, int x, int y) {
  return c.edge[(size_t)x * (c.jmax + 1) + y];
}

// L1
__global__ void k_l1(const hc_view c, LatBufs b) {
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int xr = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > c.jmax - 1 || xr > c.imax) return;
  if (!c.mask[(size_t)xr * c.W + y]) return;
  int x = xr;
  if (x == 1) x++;
  if (x == c.jmax) x--;
  const double t = c.tau[(size_t)x * c.W + y];
  if (t > kMft) {
    int tc = 0;
    for (int dir = 1; dir <= 8; dir++)
      if (c.tau[(size_t)(x + kLx[dir]) * c.W + (y + kLy[dir])] < kMft) tc++;
    b.wd2[L(c, x, y)] = (tc > 6) ? 0.0 : t;
  }
}

// L2
__global__ void k_l2(const hc_view c, LatBufs b) {
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 2 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > c.imax - 1 || x > c.jmax - 1) return;
  const double w = b.wd2[L(c, x, y)];
  EDG(c, x, y) = -9999;
  if (w < kMft) {
    const double a = b.wd2[L(c, x, y - 1)], bb = b.wd2[L(c, x - 1, y)],
                 cc = b.wd2[L(c, x + 1, y)], dd = b.wd2[L(c, x, y + 1)];
    if (a > kMft || bb > kMft || cc > kMft || dd > kMft) EDG(c, x, y) = 0;
    if (a > kMft && bb > kMft && cc > kMft && dd > kMft) {
      EDG(c, x, y) = -9999;
      c.edge2[(size_t)x * (c.jmax + 1) + y] = -9999;
    }
    b.up[U(c, 2 * x, 2 * y)] = 0;
    b.up[U(c, 2 * x, 2 * y - 1)] = 0;
    b.up[U(c, 2 * x - 1, 2 * y)] = 0;
    b.up[U(c, 2 * x - 1, 2 * y - 1)] = 0;
  }
  if (w >= kMft) {
    b.up[U(c, 2 * x, 2 * y)] = 1;
    b.up[U(c, 2 * x, 2 * y - 1)] = 1;
    b.up[U(c, 2 * x - 1, 2 * y)] = 1;
    b.up[U(c, 2 * x - 1, 2 * y - 1)] = 1;
  }
}

// L3: 0 -> 2 next to a wet cell (writes never create a 1, so the in-place
// update reads the same as the reference's sweep)
__global__ void k_l3(const hc_view c, LatBufs b) {
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 2 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > 2 * c.imax - 1 || x > 2 * c.jmax - 1) return;
  b.upe[U(c, x, y)] = 0;
  if (b.up[U(c, x, y)] == 0)
    if (b.up[U(c, x, y - 1)] == 1 || b.up[U(c, x - 1, y)] == 1 || b.up[U(c, x + 1, y)] == 1 ||
        b.up[U(c, x, y + 1)] == 1)
      b.up[U(c, x, y)] = 2;
}

// L4
__global__ void k_l4(const hc_view c, LatBufs b) {
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 2 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > 2 * c.imax - 1 || x > 2 * c.jmax - 1) return;
  if (b.up[U(c, x, y)] != 2) return;
  int wet = 0, dry = 0, ecc = 1;
  for (int dir = 1; dir <= 7; dir += 2) {
    const int v = b.up[U(c, x + kLx[dir], y + kLy[dir])];
    if (v == 1) wet += 1;
    if (v == 0) dry += 1;
    if (v == 2) ecc += 1;
  }
  if (ecc > 3) dry += ecc - 2;
  b.upe[U(c, x, y)] = wet - dry;
}

// L5
__global__ void k_l5(const hc_view c, LatBufs b) {
  const int y = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > c.imax || x > c.jmax) return;
  double& e = EDG(c, x, y);
  if (e == 0) {
    e = (double)(b.upe[U(c, 2 * x, 2 * y)] + b.upe[U(c, 2 * x, 2 * y - 1)] +
                 b.upe[U(c, 2 * x - 1, 2 * y)] + b.upe[U(c, 2 * x - 1, 2 * y - 1)]);
    if (e > 2) e = 2;
    if (e < -2) e = -2;
  }
}

// whether neighbour dir of (x,y) joins the smoothing mean (:5061-5196)
__device__ __forceinline__ bool joins(const hc_view& c, const LatBufs& b, int x, int y, int dir) {
  const int dx = kLx[dir], dy = kLy[dir];
  const double* w = b.wd2;
  if ((abs(dx) + abs(dy)) != 2) {
    if (dx == 1 && dy == 0) return w[L(c, x + 1, y - 1)] > kMft || w[L(c, x + 1, y + 1)] > kMft;
    if (dx == 0 && dy == 1) return w[L(c, x + 1, y + 1)] > kMft || w[L(c, x - 1, y + 1)] > kMft;
    if (dx == -1 && dy == 0) return w[L(c, x - 1, y - 1)] > kMft || w[L(c, x - 1, y + 1)] > kMft;
    if (dx == 0 && dy == -1) return w[L(c, x - 1, y - 1)] > kMft || w[L(c, x + 1, y - 1)] > kMft;
  } else {
    if (dx == -1 && dy == -1) return w[L(c, x, y - 1)] < kMft || w[L(c, x - 1, y)] < kMft;
    if (dx == 1 && dy == -1) return w[L(c, x, y - 1)] < kMft || w[L(c, x + 1, y)] < kMft;
    if (dx == 1 && dy == 1) return w[L(c, x + 1, y)] < kMft || w[L(c, x, y + 1)] < kMft;
    if (dx == -1 && dy == 1) return w[L(c, x, y + 1)] < kMft || w[L(c, x - 1, y)] < kMft;
  }
  return false;
}

// one smoothing value at row x of column y (edge > -9999 there); returns
// whether edge_temp gets written and the value
__device__ bool l6_value(const hc_view& c, const LatBufs& b, int x, int y, bool late, double& v) {
  double mean = 0, num = 0;
  mean += EDG(c, x, y);
  num++;
  double mws0 = 0;
  bool mws0_done = false;
  for (int dir = 1; dir <= 8; dir++) {
    const int x2 = x + kLx[dir], y2 = y + kLy[dir];
    const double e2 = EDG(c, x2, y2);
    if (!(e2 > -9999 && b.wd2[L(c, x2, y2)] < kMft)) continue;
    bool take;
    if (late) {
      if (!mws0_done) {
        mws0 = mean_ws_elev_dev(c, x, y);
        mws0_done = true;
      }
      take = mean_ws_elev_dev(c, x2, y2) > mws0 && joins(c, b, x, y, dir);
    } else {
      take = joins(c, b, x, y, dir);
    }
    if (take) {
      mean += e2;
      num++;
    }
  }
  bool write = false;
  if (mean != 0) {
    v = mean / num;
    write = true;
  }
  if (x < 3 || x > (c.jmax - 3) || y < 3 || y > (c.imax - 3)) {
    v = 0;
    write = true;
  }
  return write;
}

// L6a: entries of rows 3..jmax-2 (unique writers)
__global__ void k_l6_inner(const hc_view c, LatBufs b, int late) {
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 3 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > c.imax - 1 || x > c.jmax - 2) return;
  if (!c.mask[(size_t)x * c.W + y]) return;
  b.et[L(c, x, y)] = 0;
  if (EDG(c, x, y) > -9999) {
    double v;
    if (l6_value(c, b, x, y, late != 0, v)) b.et[L(c, x, y)] = v;
  }
}

// L6b: entries of rows 1, 2, jmax-1, jmax of each column, in loop order
__global__ void k_l6_border(const hc_view c, LatBufs b, int late) {
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  if (y > c.imax - 1) return;
  const int J = c.jmax;
  const int rows[4] = {1, 2, J - 1, J};
  for (int r = 0; r < 4; r++) {
    const int xr = rows[r];
    if (xr < 1 || xr > c.imax) continue;
    if (r >= 2 && xr <= 2) continue;  // tiny grids: rows already handled
    if (!c.mask[(size_t)xr * c.W + y]) continue;
    b.et[L(c, xr, y)] = 0;
    int x = xr;
    if (x == 1) x++;
    if (x == J) x--;
    if (EDG(c, x, y) > -9999) {
      double v;
      if (l6_value(c, b, x, y, late != 0, v)) b.et[L(c, x, y)] = v;
    }
  }
}

// L6 copy: edge = edge_temp for every entry (its own row)
__global__ void k_l6_copy(const hc_view c, LatBufs b) {
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > c.imax - 1 || x > c.imax) return;
  if (!c.mask[(size_t)x * c.W + y]) return;
  if (EDG(c, x, y) > -9999) EDG(c, x, y) = b.et[L(c, x, y)];
}

// L7
__global__ void k_l7(const hc_view c) {
  const int y = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > c.imax || x > c.jmax) return;
  double e = EDG(c, x, y);
  if (e > -9999) {
    if (e > 0) e = 0;
    e = 0 - e;
    e = 1 / ((2.131 * pow(e, -1.0794)) * c.p.DX);
  }
  if (c.h[(size_t)x * c.W + y] > c.p.water_depth_erosion_threshold && e == -9999) e = 0;
  EDG(c, x, y) = e;
}

// L8a: edge_temp of the cross-channel smoothing.  The reference turns a wet
// cell's -9999 into 0 right before every read of it; every read here uses
// that value, and the conversions are written back (all writers agree).
__device__ __forceinline__ double eff_edge(const hc_view& c, const LatBufs& b, int x, int y) {
  double e = EDG(c, x, y);
  if (b.wd2[L(c, x, y)] > kMft && e == -9999) {
    EDG(c, x, y) = 0;
    e = 0;
  }
  return e;
}

__device__ void l8_entry(const hc_view& c, LatBufs& b, int xr, int y) {
  b.et[L(c, xr, y)] = 0;
  int x = xr;
  if (x == 1) x++;
  if (x == c.jmax) x--;
  const double e0 = eff_edge(c, b, x, y);
  if (e0 > -9999 && b.wd2[L(c, x, y)] > kMft) {
    double mean = 0;
    int num = 0;
    for (int dir = 1; dir <= 8; dir += 2) {
      const double e2 = eff_edge(c, b, x + kLx[dir], y + kLy[dir]);
      if (e2 > -9999) {
        mean += e2;
        num++;
      }
    }
    b.et[L(c, x, y)] = mean / num;
  }
}

__global__ void k_l8_inner(const hc_view c, LatBufs b) {
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 3 + blockIdx.y * blockDim.y + threadIdx.y;
  if (y > c.imax - 1 || x > c.jmax - 2) return;
  if (!c.mask[(size_t)x * c.W + y]) return;
  l8_entry(c, b, x, y);
}

__global__ void k_l8_border(const hc_view c, LatBufs b) {
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  if (y > c.imax - 1) return;
  const int J = c.jmax;
  const int rows[4] = {1, 2, J - 1, J};
  for (int r = 0; r < 4; r++) {
    const int xr = rows[r];
    if (xr < 1 || xr > c.imax) continue;
    if (r >= 2 && xr <= 2) continue;
    if (!c.mask[(size_t)xr * c.W + y]) continue;
    l8_entry(c, b, xr, y);
  }
}

// L8b: copy where wet, and the largest change (one writer per target row;
// the bumped duplicates of rows 2 and jmax-1 see no change the second time)
__global__ void k_l8_copy(const hc_view c, LatBufs b) {
  __shared__ double wmax[8];
  const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int x = 2 + blockIdx.y * blockDim.y + threadIdx.y;
  double m = 0;
  if (y <= c.imax - 1 && x <= c.jmax - 1) {
    bool visited = c.mask[(size_t)x * c.W + y] != 0;
    if (x == 2 && c.mask[(size_t)1 * c.W + y]) visited = true;
    if (x == c.jmax - 1 && c.jmax <= c.imax && c.mask[(size_t)c.jmax * c.W + y]) visited = true;
    if (visited) {
      const double e = EDG(c, x, y);
      if (e > -9999 && b.wd2[L(c, x, y)] > kMft) {
        const double t = b.et[L(c, x, y)];
        m = fabs(e - t);
        if (!(m == m)) m = 0;  // a NaN change never raises the reference's max
        EDG(c, x, y) = t;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = smax(m, __shfl_xor_sync(0xffffffffu, m, o));
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  if ((t & 31) == 0) wmax[t >> 5] = m;
  __syncthreads();
  if (t == 0) {
    double bm = 0;
    for (int w = 0; w < (int)(blockDim.x * blockDim.y) / 32; w++) bm = smax(bm, wmax[w]);
    if (bm > 0) atomic_max_pos((unsigned long long*)b.diff, bm);
  }
}

}  // namespace

size_t lateral_scratch_bytes(int imax, int jmax) {
  const size_t n1 = (size_t)(jmax + 1) * (imax + 1);
  const size_t n2 = (size_t)(2 * (jmax + 1)) * (2 * (imax + 1));
  return 2 * n1 * 8 + 2 * n2 * 4 + 256;
}

hc_status run_lateral(hc_ctx* c) {
  const hc_view& v = c->v;
  if (v.imax != v.jmax) return hc_fail(c, HC_ERR_UNSUPPORTED, "lateral3 needs a square grid");
  extern double* lateral_buffer(hc_ctx*);
  char* base = (char*)lateral_buffer(c);
  const size_t n1 = (size_t)(v.jmax + 1) * (v.imax + 1);
  const size_t n2 = (size_t)(2 * (v.jmax + 1)) * (2 * (v.imax + 1));
  LatBufs b;
  b.et = (double*)base;
  b.wd2 = b.et + n1;
  b.up = (int*)(b.wd2 + n1);
  b.upe = b.up + n2;
  b.diff = (double*)(b.upe + n2);
  cudaStream_t s = c->s;
  // fresh scratch arrays per call, as the reference declares them
  cudaMemsetAsync(base, 0, 2 * n1 * 8 + 2 * n2 * 4, s);
  dim3 bl(32, 8);
  auto g = [&](int ny, int nx) { return dim3((ny + 31) / 32 > 0 ? (ny + 31) / 32 : 1, (nx + 7) / 8 > 0 ? (nx + 7) / 8 : 1); };
  const int I = v.imax, J = v.jmax;
  k_l1<<<g(J - 2, I), bl, 0, s>>>(v, b);
  k_l2<<<g(I - 2, J - 2), bl, 0, s>>>(v, b);
  k_l3<<<g(2 * I - 2, 2 * J - 2), bl, 0, s>>>(v, b);
  k_l4<<<g(2 * I - 2, 2 * J - 2), bl, 0, s>>>(v, b);
  k_l5<<<g(I, J), bl, 0, s>>>(v, b);
  const double esp = v.p.edge_smoothing_passes;
  for (int n = 1; n <= esp + v.p.downstream_shift; n++) {
    const int late = n > esp;
    k_l6_inner<<<g(I - 2, J - 4), bl, 0, s>>>(v, b, late);
    k_l6_border<<<(I + 127) / 128, 128, 0, s>>>(v, b, late);
    k_l6_copy<<<g(I - 2, I), bl, 0, s>>>(v, b);
  }
  k_l7<<<g(I, J), bl, 0, s>>>(v);
  double diff = 0;
  int guard = 0;
  do {
    cudaMemsetAsync(b.diff, 0, sizeof(double), s);
    k_l8_inner<<<g(I - 2, J - 4), bl, 0, s>>>(v, b);
    k_l8_border<<<(I + 127) / 128, 128, 0, s>>>(v, b);
    k_l8_copy<<<g(I - 2, J - 2), bl, 0, s>>>(v, b);
    cudaError_t e = cudaMemcpyAsync(&diff, b.diff, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return hc_cuda(c, e, "lateral3");
    if (++guard > 10000000) return hc_fail(c, HC_ERR_TIMEOUT, "lateral3 did not converge");
  } while (diff > v.p.lateral_cross_channel_smoothing);
  return HC_OK;
}
