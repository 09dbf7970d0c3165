// Test driver: the library's integer-pipe division (ddiv_rn, ddiv_by in
// hc_internal.cuh) against the hardware's IEEE division, bit for bit, over
// several input families, with divisors prepared on the device and on the
// host; and the throughput of both.  Built by
// test_gpu_arith.py with the library's own compiler flags.
#include <cstdint>
#include <cstring>

#include "../hail-caesar_gb300/csrc/hc_internal.cuh"

namespace {

__device__ __forceinline__ unsigned long long mix(unsigned long long x) {  // splitmix64
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ double mk(unsigned long long sign, int e, unsigned long long m) {
  return __longlong_as_double(
      (long long)((sign << 63) | ((unsigned long long)(e & 0x7ff) << 52) | (m & ((1ull << 52) - 1))));
}

__device__ void pair(int mode, unsigned long long k, double& a, double& b) {
  const unsigned long long r1 = mix(k), r2 = mix(k ^ 0xabcdef12345ull), r3 = mix(k * 7 + 3);
  switch (mode) {
    case 0:  // any bit patterns: zeros, subnormals, infinities, NaNs included
      a = __longlong_as_double((long long)r1);
      b = __longlong_as_double((long long)r2);
      break;
    case 1:  // normal operands, quotients across the whole normal range
      a = mk(r3 & 1, 1 + (int)(r1 >> 53) % 2046, r1);
      b = mk((r3 >> 1) & 1, 1 + (int)(r2 >> 53) % 2046, r2);
      break;
    case 2: {  // significands at the ends of their range
      const unsigned long long ma = (r3 & 4) ? (r1 & 0xffff) : ((1ull << 52) - 1 - (r1 & 0xffff));
      const unsigned long long mb = (r3 & 8) ? (r2 & 0xffff) : ((1ull << 52) - 1 - (r2 & 0xffff));
      a = mk(r3 & 1, 1023 + (int)(r1 >> 58) - 32, ma);
      b = mk((r3 >> 1) & 1, 1023 + (int)(r2 >> 58) - 32, mb);
      break;
    }
    case 3: {  // quotients at or next to small integers and simple fractions
      b = mk(0, 1000 + (int)(r2 >> 58), r2);
      const double m = (double)(1 + (r1 >> 56));
      const double p = b * m;
      const long long d = (long long)(r3 % 5) - 2;
      a = __longlong_as_double(__double_as_longlong(p) + d);
      break;
    }
    case 4: {  // quotients at the edges of the normal range
      const int eb = 1 + (int)(r2 >> 53) % 2046;
      const int t = (int)(r3 % 8);
      const int target = (t < 4) ? (t - 1) : (2044 + (t - 4));  // -1..2, 2044..2047
      int ea = target + eb - 1023;
      if (ea < 1) ea = 1;
      if (ea > 2046) ea = 2046;
      a = mk(r3 >> 63, ea, r1);
      b = mk(0, eb, r2);
      break;
    }
    case 5: {  // the model's magnitudes: depths, discharges, volumes
      a = mk(r3 & 1, 1023 - 30 + (int)(r1 >> 59), r1);
      b = mk(0, 1023 - 20 + (int)(r2 >> 59), r2);
      break;
    }
    default: {  // signed zero and subnormal dividends, any divisors
      a = mk(r3 & 1, 0, (r3 & 2) ? 0ull : r1);
      b = (r3 & 4) ? __longlong_as_double((long long)r2) : mk(r2 >> 63, 1 + (int)(r2 >> 53) % 2046, r2);
    }
  }
}

__global__ void k_check(unsigned long long n, unsigned long long seed, int mode,
                        unsigned long long* bad, double* first) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    double a, b;
    pair(mode, k + seed * 0x100000000ull, a, b);
    const double x = ddiv_rn(a, b), y = __ddiv_rn(a, b);
    const bool same = __double_as_longlong(x) == __double_as_longlong(y) ||
                      (disnan(x) && disnan(y));
    if (!same && atomicAdd(bad, 1ull) == 0) {
      first[0] = a;
      first[1] = b;
      first[2] = x;
      first[3] = y;
    }
  }
}

// quotients by divisors prepared on the host (exact reciprocal), as the
// library prepares DX and the Einstein constants
__global__ void k_check_prepared(unsigned long long n, unsigned long long seed,
                                 const hc_divisor* tab, int ntab, unsigned long long* bad,
                                 double* first) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long r1 = mix(k + seed * 0x100000000ull);
    const hc_divisor& d = tab[(r1 >> 40) % ntab];
    const double a = ((r1 & 7) == 0)   ? __longlong_as_double((long long)mix(r1))
                     : ((r1 & 15) == 1) ? mk(r1 >> 63, 0, 0)  // signed zeros
                                        : mk(r1 >> 63, 1023 - 60 + (int)((r1 >> 52) & 127), mix(r1));
    const double x = ddiv_by(a, d), y = __ddiv_rn(a, d.b);
    const bool same = __double_as_longlong(x) == __double_as_longlong(y) ||
                      (disnan(x) && disnan(y));
    if (!same && atomicAdd(bad, 1ull) == 0) {
      first[0] = a;
      first[1] = d.b;
      first[2] = x;
      first[3] = y;
    }
  }
}

// the integer-pipe cube against the FP64 one; the first 64 arguments where
// they differ are kept with both results (the caller decides which one is
// correctly rounded)
__global__ void k_check_cube(unsigned long long n, unsigned long long seed, int mode,
                             unsigned long long* bad, double* keep) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long r = mix(k + seed * 0x100000000ull);
    double h;
    if (mode == 0) h = __longlong_as_double((long long)r);               // any bit pattern
    else if (mode == 1) h = mk(0, 1023 - 40 + (int)((r >> 52) % 48), r);  // depths
    else h = mk(0, 1023 - 20 + (int)((r >> 52) % 30), (r >> 35) << 35);   // short significands
    const double x = icube_rn(h), y = cube_rn(h);
    const bool same = __double_as_longlong(x) == __double_as_longlong(y) ||
                      (disnan(x) && disnan(y));
    if (!same) {
      const unsigned long long i = atomicAdd(bad, 1ull);
      if (i < 64) {
        keep[3 * i] = h;
        keep[3 * i + 1] = x;
        keep[3 * i + 2] = y;
      }
    }
  }
}

// the integer-pipe float <-> double conversions against the instructions
__global__ void k_check_conv(unsigned long long n, unsigned long long seed,
                             unsigned long long* bad, double* first) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long r = mix(k + seed * 0x100000000ull);
    // doubles: any bits, and values near the float range and its roundings
    const double x = (k & 1) ? __longlong_as_double((long long)r)
                             : mk(r >> 63, 1023 - 130 + (int)((r >> 52) % 260), r);
    const float a = d2f_i(x), b = __double2float_rn(x);
    const float f = __uint_as_float((unsigned)(r >> 17));
    const double p = f2d_i(f), q = (double)f;
    const bool same1 = __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
    const bool same2 = __double_as_longlong(p) == __double_as_longlong(q) || (p != p && q != q);
    if (!(same1 && same2) && atomicAdd(bad, 1ull) == 0) {
      first[0] = x;
      first[1] = (double)f;
    }
  }
}

// the integer-pipe square root against the hardware's
__global__ void k_check_sqrt(unsigned long long n, unsigned long long seed, int mode,
                             unsigned long long* bad, double* first) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long r = mix(k + seed * 0x100000000ull);
    double x;
    if (mode == 0) x = __longlong_as_double((long long)r);            // any bit pattern
    else if (mode == 1) x = mk(0, 1 + (int)((r >> 52) % 2046), r);    // positive normal
    else {                                                            // squares and neighbours
      const double q = (double)(r >> 40) + 1.0;
      x = __longlong_as_double(__double_as_longlong(q * q) + (long long)(r & 3) - 1);
    }
    const double a = isqrt_rn(x), b = sqrt(x);
    const bool same = __double_as_longlong(a) == __double_as_longlong(b) || (disnan(a) && disnan(b));
    if (!same && atomicAdd(bad, 1ull) == 0) {
      first[0] = x;
      first[1] = a;
      first[2] = b;
    }
  }
}

// throughput: each thread divides independent operands kIter times
template <bool kInt>
__global__ void k_time(const double* in, double* out, int iters) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double a = in[t & 1023] + t * 1e-9, b = in[(t + 7) & 1023] + 1.5;
  double acc = 0;
  for (int k = 0; k < iters; k++) {
    const double q = kInt ? ddiv_rn(a, b) : __ddiv_rn(a, b);
    acc = acc + q;
    a = q + 1.25;  // the next quotient depends on this one
  }
  out[t] = acc;
}

}  // namespace

extern "C" int arith_check(unsigned long long n, unsigned long long seed, int mode,
                           unsigned long long* bad, double* first) {
  unsigned long long* d_bad;
  double* d_first;
  if (cudaMalloc(&d_bad, 8) != cudaSuccess || cudaMalloc(&d_first, 32) != cudaSuccess) return 1;
  cudaMemset(d_bad, 0, 8);
  cudaMemset(d_first, 0, 32);
  k_check<<<152 * 16, 256>>>(n, seed, mode, d_bad, d_first);
  cudaMemcpy(bad, d_bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(first, d_first, 32, cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  cudaFree(d_bad);
  cudaFree(d_first);
  return e == cudaSuccess ? 0 : 2;
}

extern "C" int arith_check_cube(unsigned long long n, unsigned long long seed, int mode,
                                unsigned long long* bad, double* keep) {
  unsigned long long* d_bad;
  double* d_keep;
  if (cudaMalloc(&d_bad, 8) != cudaSuccess || cudaMalloc(&d_keep, 3 * 64 * 8) != cudaSuccess)
    return 1;
  cudaMemset(d_bad, 0, 8);
  cudaMemset(d_keep, 0, 3 * 64 * 8);
  k_check_cube<<<152 * 16, 256>>>(n, seed, mode, d_bad, d_keep);
  cudaMemcpy(bad, d_bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(keep, d_keep, 3 * 64 * 8, cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  cudaFree(d_bad);
  cudaFree(d_keep);
  return e == cudaSuccess ? 0 : 2;
}

extern "C" int arith_check_conv(unsigned long long n, unsigned long long seed,
                                unsigned long long* bad, double* first) {
  unsigned long long* d_bad;
  double* d_first;
  if (cudaMalloc(&d_bad, 8) != cudaSuccess || cudaMalloc(&d_first, 32) != cudaSuccess) return 1;
  cudaMemset(d_bad, 0, 8);
  cudaMemset(d_first, 0, 32);
  k_check_conv<<<152 * 16, 256>>>(n, seed, d_bad, d_first);
  cudaMemcpy(bad, d_bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(first, d_first, 32, cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  cudaFree(d_bad);
  cudaFree(d_first);
  return e == cudaSuccess ? 0 : 2;
}

extern "C" int arith_check_sqrt(unsigned long long n, unsigned long long seed, int mode,
                                unsigned long long* bad, double* first) {
  unsigned long long* d_bad;
  double* d_first;
  if (cudaMalloc(&d_bad, 8) != cudaSuccess || cudaMalloc(&d_first, 32) != cudaSuccess) return 1;
  cudaMemset(d_bad, 0, 8);
  cudaMemset(d_first, 0, 32);
  k_check_sqrt<<<152 * 16, 256>>>(n, seed, mode, d_bad, d_first);
  cudaMemcpy(bad, d_bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(first, d_first, 32, cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  cudaFree(d_bad);
  cudaFree(d_first);
  return e == cudaSuccess ? 0 : 2;
}

// the host preparation of a divisor (exact floor(2^116/mb))
static hc_divisor prepare(double b) {
  unsigned long long B;
  memcpy(&B, &b, 8);
  const unsigned long long H52 = 1ull << 52;
  hc_divisor d;
  d.b = b;
  d.eb = (int)(B >> 52) & 0x7ff;
  d.ok = d.eb != 0 && d.eb != 0x7ff;
  d.mb = (B & (H52 - 1)) | H52;
  d.V = (d.mb == H52) ? 0 : (unsigned long long)(((unsigned __int128)1 << 116) / d.mb);
  return d;
}

extern "C" int arith_check_prepared(unsigned long long n, unsigned long long seed,
                                    unsigned long long* bad, double* first) {
  const int ntab = 4099;
  hc_divisor* h = new hc_divisor[ntab];
  unsigned long long x = seed;
  for (int k = 0; k < ntab; k++) {
    x = x * 6364136223846793005ull + 1442695040888963407ull;
    double b;
    if (k < 8) {
      const double fixed[8] = {1.0, 2.0, 10.0, 20.0, 9.81, 0.5, 3.0, 1e-3};
      b = fixed[k];
    } else {
      const unsigned long long e = 1023 - 40 + ((x >> 33) % 80);
      const unsigned long long m = (k % 5 == 0) ? ((x >> 11) & 0xff) : (x >> 12);
      const unsigned long long bits = (e << 52) | (m & ((1ull << 52) - 1));
      memcpy(&b, &bits, 8);
    }
    h[k] = prepare(b);
  }
  hc_divisor* tab;
  unsigned long long* d_bad;
  double* d_first;
  if (cudaMalloc(&tab, ntab * sizeof(hc_divisor)) != cudaSuccess ||
      cudaMalloc(&d_bad, 8) != cudaSuccess || cudaMalloc(&d_first, 32) != cudaSuccess)
    return 1;
  cudaMemcpy(tab, h, ntab * sizeof(hc_divisor), cudaMemcpyHostToDevice);
  cudaMemset(d_bad, 0, 8);
  cudaMemset(d_first, 0, 32);
  k_check_prepared<<<152 * 16, 256>>>(n, seed, tab, ntab, d_bad, d_first);
  cudaMemcpy(bad, d_bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(first, d_first, 32, cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  cudaFree(tab);
  cudaFree(d_bad);
  cudaFree(d_first);
  delete[] h;
  return e == cudaSuccess ? 0 : 2;
}

// divisions per second of each kind (ms for `iters` divisions per thread)
extern "C" int arith_time(int iters, float* ms_native, float* ms_int) {
  const int blocks = 152 * 8, threads = 256;
  double *in, *out;
  if (cudaMalloc(&in, 1024 * 8) != cudaSuccess ||
      cudaMalloc(&out, (size_t)blocks * threads * 8) != cudaSuccess)
    return 1;
  double h[1024];
  for (int k = 0; k < 1024; k++) h[k] = 0.1 + k * 0.37;
  cudaMemcpy(in, h, sizeof h, cudaMemcpyHostToDevice);
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  k_time<false><<<blocks, threads>>>(in, out, 16);  // warm-up
  k_time<true><<<blocks, threads>>>(in, out, 16);
  cudaEventRecord(e0);
  k_time<false><<<blocks, threads>>>(in, out, iters);
  cudaEventRecord(e1);
  k_time<true><<<blocks, threads>>>(in, out, iters);
  cudaEventRecord(e2);
  cudaEventSynchronize(e2);
  cudaEventElapsedTime(ms_native, e0, e1);
  cudaEventElapsedTime(ms_int, e1, e2);
  const cudaError_t e = cudaGetLastError();
  cudaFree(in);
  cudaFree(out);
  return e == cudaSuccess ? 0 : 2;
}
