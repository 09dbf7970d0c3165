// depth_update (src/catchmentmodel/LSDCatchmentModel.cpp:3259-3299) on
// device buffers the caller owns, with no device allocation at all.
//
// Who needs it: a caller that keeps the reference's TNT arrays mirrored in
// device memory of its own (a host program with a fixed device-memory budget
// already spent, or one that shares the GPU with other streams) cannot afford
// hc_create's buffers, and cannot let a call allocate: cudaMalloc can fail at
// the budget, and cudaFree waits for the whole device, stalling every other
// stream.  The one piece of working memory the update needs -- the per-column
// maxima that the reference keeps in `tempmaxdepth` and combines into
// `maxdepth` -- lives in a fixed array of this library's module instead.
//
// Scratch: g_depth_scratch, 1 + HC_DEPTH_NOALLOC_MAX_COLS doubles (128 KiB).
//   element 0     done counter (its bits, as an unsigned 64-bit integer);
//                 must be zero when a call starts.  It is zero when the module
//                 loads and every call leaves it at zero.
//   element 1 + y maximum depth of column y of the current call; written by
//                 the call before it is read, so it needs no clearing.
// Every call on a device shares this one array: two calls in flight at the
// same time on that device (on different streams, or from different threads)
// race on it and corrupt each other's maxdepth.  Order calls on one stream.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/hc_gpu.h"

namespace {

constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_depth_scratch[1 + HC_DEPTH_NOALLOC_MAX_COLS];

std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};

hc_status say(char* err, size_t len, hc_status st, const char* fmt, ...) {
  if (err && len) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, len, fmt, ap);
    va_end(ap);
  }
  return st;
}

// One block per column y (the reference's outer loop); the block's threads
// take the column's down_scan entries x in turn.  The last block to finish
// combines the column maxima.
__global__ void __launch_bounds__(256)
    k_depth_update_noalloc(int imax, int jmax, double DX, double dt,
                           const int32_t* __restrict__ down_scan,
                           const double* __restrict__ elev, const double* __restrict__ qx,
                           const double* __restrict__ qy, const double* __restrict__ qxs,
                           const double* __restrict__ qys, double* __restrict__ h,
                           double* __restrict__ vs, double* __restrict__ maxdepth,
                           double* scratch) {
  __shared__ int end;
  __shared__ double warp_max[8];
  __shared__ bool last;
  const int y = 1 + blockIdx.x;
  const int t = threadIdx.x;
  const size_t W = (size_t)jmax + 2;
  const int32_t* col = down_scan + (size_t)y * (imax + 2);
  // the column's list ends at its first entry that is not positive
  // (the reference's `while (down_scan[y][inc] > 0)`); entries 1..imax+1
  if (t == 0) end = imax + 2;
  __syncthreads();
  for (int k = 1 + t; k <= imax + 1; k += blockDim.x)
    if (col[k] <= 0) atomicMin(&end, k);
  __syncthreads();
  const int n_end = end;
  double m = 0;
  for (int k = 1 + t; k < n_end; k += blockDim.x) {
    const int x = col[k];
    if (x > imax) continue;  // not a row of the grid
    const size_t cell = (size_t)x * W + y;
    double d = h[cell];
    d += dt * (qx[cell + W] - qx[cell] + qy[cell + 1] - qy[cell]) / DX;
    if (vs) vs[cell] += dt * (qxs[cell + W] - qxs[cell] + qys[cell + 1] - qys[cell]) / DX;
    if (d > 0) {
      if (elev[cell] == -9999) d = 0;
      if (d > m) m = d;
    }
    h[cell] = d;
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((t & 31) == 0) warp_max[t >> 5] = m;
  __syncthreads();
  unsigned long long* done = reinterpret_cast<unsigned long long*>(scratch);
  if (t == 0) {
    double b = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) b = fmax(b, warp_max[w]);
    scratch[y] = b;
    __threadfence();
    last = (atomicAdd(done, 1ull) == (unsigned long long)gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double g = 0;
  for (int c = 1 + t; c <= jmax; c += blockDim.x) g = fmax(g, __ldcg(&scratch[c]));
  for (int o = 16; o > 0; o >>= 1) g = fmax(g, __shfl_xor_sync(0xffffffffu, g, o));
  __syncthreads();
  if ((t & 31) == 0) warp_max[t >> 5] = g;
  __syncthreads();
  if (t == 0) {
    double b = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) b = fmax(b, warp_max[w]);
    *maxdepth = b;
    atomicExch(done, 0ull);  // the next call starts from zero
  }
}

// Set-up, once per device, with that device current: the scratch array's
// device address.  The first call on a device does this look-up, so that
// first call should come before any stream capture begins.
hc_status scratch_of_current_device(double** out, char* err, size_t len) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return say(err, len, HC_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return say(err, len, HC_ERR_UNSUPPORTED, "device ordinal %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    double* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_depth_scratch);
    if (e != cudaSuccess)
      return say(err, len, HC_ERR_CUDA, "cudaGetSymbolAddress(scratch) on device %d: %s", dev,
                 cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return HC_OK;
}

}  // namespace

extern "C" hc_status hc_depth_update_noalloc(int32_t imax, int32_t jmax, double DX,
                                             double flow_timestep, const int32_t* down_scan,
                                             const double* elev, const double* qx,
                                             const double* qy, const double* qxs,
                                             const double* qys, double* water_depth,
                                             double* Vsusptot, double* maxdepth, void* stream,
                                             char* err, size_t err_len) {
  if (err && err_len) err[0] = 0;
  if (imax < 1 || jmax < 1)
    return say(err, err_len, HC_ERR_ARG, "imax %d and jmax %d must be at least 1", imax, jmax);
  if (jmax > HC_DEPTH_NOALLOC_MAX_COLS)
    return say(err, err_len, HC_ERR_ARG,
               "jmax %d exceeds HC_DEPTH_NOALLOC_MAX_COLS (%d), the size of the fixed scratch "
               "array; use hc_depth_update", jmax, HC_DEPTH_NOALLOC_MAX_COLS);
  if (!(DX > 0))
    return say(err, err_len, HC_ERR_ARG, "DX must be positive");
  if (!down_scan || !elev || !qx || !qy || !water_depth || !maxdepth)
    return say(err, err_len, HC_ERR_ARG, "null buffer");
  if (Vsusptot && (!qxs || !qys))
    return say(err, err_len, HC_ERR_ARG, "Vsusptot needs qxs and qys");
  double* scratch = nullptr;
  hc_status st = scratch_of_current_device(&scratch, err, err_len);
  if (st != HC_OK) return st;
  k_depth_update_noalloc<<<jmax, 256, 0, (cudaStream_t)stream>>>(
      imax, jmax, DX, flow_timestep, down_scan, elev, qx, qy, qxs, qys, water_depth, Vsusptot,
      maxdepth, scratch);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return say(err, err_len, HC_ERR_CUDA, "depth_update launch: %s", cudaGetErrorString(e));
  return HC_OK;
}
