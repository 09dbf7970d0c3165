// The C ABI of libhc_gpu (include/hc_gpu.h): context life cycle, field
// transfers in the reference's layouts, the member-level entry points, and
// hc_run, which executes whole iterations of the reference's main loop from a
// CUDA graph with the driver's scalar logic on the device.

#include "hc_internal.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

size_t lateral_scratch_bytes(int imax, int jmax);

// ------------------------------------------------------------------ errors
hc_status hc_fail(hc_ctx* c, hc_status st, const char* fmt, ...) {
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof c->err, fmt, ap);
    va_end(ap);
  }
  return st;
}

hc_status hc_cuda(hc_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return HC_OK;
  return hc_fail(c, HC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define HC_TRY(expr)                         \
  do {                                       \
    hc_status st_ = (expr);                  \
    if (st_ != HC_OK) return st_;            \
  } while (0)
#define HC_CU(expr, what) HC_TRY(hc_cuda(c, (expr), what))

namespace {

struct Extra {
  double* lateral;  // lateral3 scratch
  float* h_rain; int h_rain_rows, h_rain_cols;
  std::vector<hc_step_record> dummy;
};

// per-context side allocations not in hc_view
std::vector<std::pair<hc_ctx*, Extra>>& extras() {
  static std::vector<std::pair<hc_ctx*, Extra>> e;
  return e;
}
Extra& extra(hc_ctx* c) {
  for (auto& p : extras())
    if (p.first == c) return p.second;
  extras().push_back({c, Extra{}});
  return extras().back().second;
}
void drop_extra(hc_ctx* c) {
  auto& e = extras();
  for (size_t k = 0; k < e.size(); k++)
    if (e[k].first == c) {
      e.erase(e.begin() + k);
      return;
    }
}

__global__ void k_fill_d(double* a, size_t n, double v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    a[i] = v;
}
__global__ void k_fill_i(int32_t* a, size_t n, int32_t v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    a[i] = v;
}
__global__ void k_fill_u64(unsigned long long* a, size_t n, unsigned long long v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    a[i] = v;
}

__global__ void k_set_max_ts(const hc_view c, hc_dev* d) {
  hc_scalars& s = d->s;
  const hc_params& p = c.p;
  s.input_output_difference = fabs(s.waterinput - s.waterOut);
  auto cfl = [&]() { return p.courant_number * (p.DX / sqrt(9.81 * (s.maxdepth))); };
  if (s.maxdepth <= 0.1) s.maxdepth = 0.1;
  if (s.time_step < cfl()) s.time_step = cfl();
  if (s.input_output_difference > p.in_out_difference_allowed && s.time_step > (cfl()))
    s.time_step = cfl();
}

template <class T>
hc_status dalloc(hc_ctx* c, T** p, size_t count) {
  size_t bytes = count * sizeof(T);
  if (bytes == 0) bytes = sizeof(T);
  if (c->max_bytes && c->bytes + bytes > c->max_bytes)
    return hc_fail(c, HC_ERR_NOMEM, "device allocation cap of %zu bytes exceeded", c->max_bytes);
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return hc_fail(c, HC_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  }
  c->bytes += bytes;
  return HC_OK;
}

void fill_d(hc_ctx* c, double* a, size_t n, double v) {
  if (!a || !n) return;
  k_fill_d<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, c->s>>>(a, n, v);
}
void fill_i(hc_ctx* c, int32_t* a, size_t n, int32_t v) {
  if (!a || !n) return;
  k_fill_i<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, c->s>>>(a, n, v);
}

}  // namespace

double* lateral_buffer(hc_ctx* c) { return extra(c).lateral; }

// ------------------------------------------------------------------ params
extern "C" void hc_params_default(hc_params* p, int32_t imax, int32_t jmax, double DX) {
  std::memset(p, 0, sizeof *p);
  p->imax = imax;
  p->jmax = jmax;
  p->DX = DX;
  p->courant_number = 0.7;
  p->froude_limit = 0.8;
  p->mannings = 0.04;
  p->hflow_threshold = 0.00001;
  p->edgeslope = 0.001;
  p->water_depth_erosion_threshold = 0.01;
  p->in_out_difference_allowed = 0;
  p->max_time_step = 0;
  p->ERODEFACTOR = 0.05;
  p->maxcycle = 1000;
  p->rain_data_time_step = 60;
  p->rfnum = 1;
  p->M = 0.005;
  p->rain_factor = 1;
  p->baseflow = 0.00000005;
  p->MIN_Q = 0.01;
  p->MIN_Q_MAXVAL = 1000.0;
  p->reach_input_data_timestep = 60;
  p->div_inputs = 1;
  p->active = 0.2;
  p->max_vel = 5;
  p->Csuspmax = 0.05;
  p->vegTauCrit = 100;
  p->veg_lat_restriction = 0.1;
  p->lateral_constant = 0.0000002;
  p->chann_lateral_erosion = 20.0;
  p->failureangle = 45;
  p->CREEP_RATE = 0.0025;
  const double d[10] = {0.0, 0.000065, 0.001, 0.002, 0.004, 0.008, 0.016, 0.032, 0.064, 0.128};
  const double dp[11] = {0.0, 0.05, 0.05, 0.15, 0.225, 0.25, 0.1, 0.075, 0.05, 0.05, 0.0};
  const double fv[11] = {0.0, 0.033, 0.109, 0.164, 0.237, 0.338, 0.479, 0.678, 0.959, 1.357, 0.0};
  for (int n = 0; n < 10; n++) p->d[n] = d[n];
  for (int n = 0; n < 11; n++) {
    p->dprop[n] = dp[n];
    p->fallVelocity[n] = fv[n];
    p->isSuspended[n] = (n == 1);
  }
  p->edge_smoothing_passes = 100.0;
  p->downstream_shift = 5.0;
  p->lateral_cross_channel_smoothing = 0.0001;
  p->scan_area_interval_iter = 5;
  p->in_channel_landslide_iter_interval = 10;
  p->creep_time_interval = 14400;
  p->global_landsliding_interval = 1440;
  p->creep_coeff = 0.028;
  p->LIMIT = 1;
}

extern "C" int64_t hc_field_count(const hc_params* p, hc_field f) {
  if (!p) return -1;
  const int64_t N2 = (int64_t)(p->imax + 2) * (p->jmax + 2);
  const int64_t E2 = (int64_t)(p->imax + 1) * (p->jmax + 1);
  const int64_t nrec = N2 / std::max(1, p->LIMIT);
  switch (f) {
    case HC_F_VEL_DIR: return N2 * 9;
    case HC_F_SR: case HC_F_SL: case HC_F_SU: case HC_F_SD: return N2 * 10;
    case HC_F_GRAIN: return nrec * 11;
    case HC_F_STRATA: return nrec * 10 * 11;
    case HC_F_EDGE: return E2;
    case HC_F_VEG: return E2 * 4;
    default:
      if (f >= 0 && f < HC_F_COUNT) return N2;
      return -1;
  }
}

extern "C" int32_t hc_field_elsize(hc_field f) {
  switch (f) {
    case HC_F_INDEX: case HC_F_DOWN_SCAN: case HC_F_RFAREA: return 4;
    case HC_F_INPUTPOINTS: return 1;
    default: return (f >= 0 && f < HC_F_COUNT) ? 8 : -1;
  }
}

extern "C" const char* hc_last_error(const hc_ctx* c) { return c ? c->err : "null context"; }
extern "C" void* hc_stream(hc_ctx* c) { return c ? (void*)c->s : nullptr; }

// ------------------------------------------------------------------ create
static hc_status free_all(hc_ctx* c);

hc_divisor host_divisor(double b) {
  unsigned long long B;
  std::memcpy(&B, &b, 8);
  const unsigned long long H52 = 1ull << 52;
  hc_divisor d;
  d.b = b;
  d.eb = (int)(B >> 52) & 0x7ff;
  d.ok = d.eb != 0 && d.eb != 0x7ff;
  d.mb = (B & (H52 - 1)) | H52;
  d.V = (d.mb == H52) ? 0 : (unsigned long long)(((unsigned __int128)1 << 116) / d.mb);
  return d;
}

extern "C" hc_status hc_create(const hc_params* p, size_t max_bytes, hc_ctx** out) {
  if (!p || !out) return HC_ERR_ARG;
  *out = nullptr;
  if (p->imax < 3 || p->jmax < 3 || !(p->DX > 0)) return HC_ERR_ARG;
  if (p->rfnum < 1 || p->rfnum > HC_MAX_RF) return HC_ERR_ARG;
  if (p->number_of_points < 0 || p->number_of_points > HC_MAX_POINTS) return HC_ERR_ARG;
  if (p->LIMIT < 1 || p->scan_area_interval_iter < 1 || p->in_channel_landslide_iter_interval < 1)
    return HC_ERR_ARG;
  if (p->vegetation_on) return HC_ERR_UNSUPPORTED;
  if ((double)(p->imax + 2) * (p->jmax + 2) * 5 > 2147483647.0) return HC_ERR_UNSUPPORTED;
  hc_ctx* c = new hc_ctx();
  std::memset((void*)c, 0, sizeof *c);
  c->max_bytes = max_bytes;
  hc_view& v = c->v;
  v.p = *p;
  v.rDX = 1.0 / p->DX;
  v.dxd = host_divisor(p->DX);
  v.DXf = (float)p->DX;
  v.flf = (float)p->froude_limit;
  v.act_hi = (float)(p->active * 1.5);
  v.act_lo = (float)(p->active / 4);
  {
    long long b;
    std::memcpy(&b, &p->hflow_threshold, 8);
    const long long sgn = b >> 63;
    v.thr_key = ((b & 0x7fffffffffffffffLL) ^ sgn) - sgn;  // dkey on the host
  }
  for (int n = 1; n <= 9; n++) {
    const double Di = p->d[n], g = 9.81;
    v.einA[n] = (2650 - 1000) * Di;
    v.einS[n] = std::sqrt(1000 / ((2250 - 1000) * g * (Di * Di * Di)));
    v.einSd[n] = host_divisor(v.einS[n]);
  }
  v.imax = p->imax;
  v.jmax = p->jmax;
  v.W = (size_t)p->jmax + 2;
  v.N2 = (size_t)(p->imax + 2) * v.W;
  v.E2 = (size_t)(p->imax + 1) * (p->jmax + 1);
  const size_t N2 = v.N2, E2 = v.E2;
  const bool sed = !p->hydro_only;
  cudaGetDevice(&c->device);
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
  if (c->sms < 1) c->sms = 1;
  c->flow_shape = 0;
  c->tuned_key = -1;
  if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->s2, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return HC_ERR_CUDA;
  }
  c->cs = c->s;
  hc_status st = HC_OK;
#define A(ptr, n)                                    \
  if (st == HC_OK) st = dalloc(c, &(ptr), (n));
  A(v.elev, N2) A(v.h, N2) A(v.qx, N2) A(v.qy, N2) A(v.qxs, N2) A(v.qys, N2) A(v.vs, N2)
  A(v.vel, N2) A(v.tau, N2) A(v.bed, N2) A(v.man, N2) A(v.area, N2) A(v.ss, N2)
  A(v.vd, 4 * N2) A(v.index, N2) A(v.mask, N2) A(v.border, N2) A(v.rfarea, N2)
  A(v.edge, E2) A(v.edge2, E2) A(v.veg, 4 * E2)
  A(v.cin_x, (size_t)p->imax * p->jmax + 2) A(v.cin_y, (size_t)p->imax * p->jmax + 2)
  A(v.wet, N2) A(v.wet_sums, (N2 + 1023) / 1024 + 1)
  // partial sums: one per block of scan_area (32 x 8 cells) or of a grid_sum
  v.vpart_cap = (int)std::max<size_t>(
      (size_t)((p->jmax + 31) / 32) * (size_t)((p->imax + 7) / 8), 152 * 8);
  A(v.vpart, (size_t)v.vpart_cap)
  A(v.drain_pos, N2) A(v.drain_f0, N2) A(v.drain_f1, N2) A(v.drain_pend, N2) A(v.drain_dt, N2)
  A(v.drain_frac, 9 * N2) A(v.drain_multi, N2)
  A(v.drain_aux, 1)
  if (sed) {
    A(v.sflux, 40 * N2) A(v.sdirty, N2) A(v.grain, kGrainStride * N2)
    A(v.strata, kStrataStride * N2) A(v.alloc_key, N2)
    A(v.erodetot, N2) A(v.erodetot3, N2) A(v.pre, kGrainStride * N2) A(v.chains, 4 * N2)
    A(v.drain_snap, N2) A(v.ent_list, N2) A(v.ent_qs, 2 * N2)
  } else {
    A(v.erodetot, N2)
  }
  char* red = nullptr;
  A(red, erode_scratch_bytes(N2, p->imax, p->jmax))
  v.red = (double*)red;
  A(v.touched, slide_scratch_bytes(N2, std::max(p->imax, p->jmax)))
  double* lat = nullptr;
  if (sed && p->imax == p->jmax) A(lat, lateral_scratch_bytes(p->imax, p->jmax) / 8 + 1)
  A(c->dev, 1)
#undef A
  if (st != HC_OK) {
    free_all(c);
    return st;
  }
  extra(c).lateral = lat;
  v.cin_cap = p->imax * p->jmax;
  if (cudaMallocHost((void**)&c->hdev, sizeof(hc_dev)) != cudaSuccess) {
    cudaGetLastError();
    free_all(c);
    return HC_ERR_NOMEM;
  }
  // zero_values :2891-2982
  cudaStream_t s = c->s;
  for (double* a : {v.h, v.qx, v.qy, v.qxs, v.qys, v.vs, v.vel, v.tau, v.man, v.area, v.ss})
    cudaMemsetAsync(a, 0, N2 * 8, s);
  fill_d(c, v.elev, N2, -9999);
  fill_d(c, v.bed, N2, -9999);
  cudaMemsetAsync(v.vd, 0, 4 * N2 * 8, s);
  fill_i(c, v.index, N2, -9999);
  cudaMemsetAsync(v.mask, 0, N2, s);
  cudaMemsetAsync(v.border, 0, N2, s);
  fill_i(c, v.rfarea, N2, 1);
  cudaMemsetAsync(v.edge, 0, E2 * 8, s);
  cudaMemsetAsync(v.edge2, 0, E2 * 8, s);
  cudaMemsetAsync(v.veg, 0, 4 * E2 * 8, s);
  cudaMemsetAsync(v.cin_x, 0, ((size_t)p->imax * p->jmax + 2) * 4, s);
  cudaMemsetAsync(v.cin_y, 0, ((size_t)p->imax * p->jmax + 2) * 4, s);
  cudaMemsetAsync(v.erodetot, 0, N2 * 8, s);
  if (sed) {
    cudaMemsetAsync(v.sflux, 0, 40 * N2 * 8, s);
    cudaMemsetAsync(v.sdirty, 0, N2, s);
    cudaMemsetAsync(v.grain, 0, kGrainStride * N2 * 8, s);
    cudaMemsetAsync(v.strata, 0, kStrataStride * N2 * 8, s);
    cudaMemsetAsync(v.erodetot3, 0, N2 * 8, s);
    k_fill_u64<<<4096, 256, 0, s>>>(v.alloc_key, N2, ~0ull);
  }
  cudaMemsetAsync(v.red, 0, erode_scratch_bytes(N2, p->imax, p->jmax), s);
  cudaMemsetAsync(v.touched, 0, slide_scratch_bytes(N2, std::max(p->imax, p->jmax)), s);
  // scalar members at their initialisers (LSDCatchmentModel.hpp)
  hc_dev* hd = c->hdev;
  std::memset(hd, 0, sizeof *hd);
  hc_scalars& sc = hd->s;
  sc.cycle = 0;
  sc.time_step = 1;
  sc.maxdepth = 10;
  sc.erode_call = 0;
  sc.erode_mult = 1;
  sc.lateralcounter = 1;
  sc.time_1 = 1;
  sc.baseflow = p->baseflow;
  sc.grain_array_tot = 1;
  sc.creep_time = 1;
  sc.creep_time2 = 1;
  for (int n = 0; n <= HC_MAX_RF; n++) sc.j[n] = sc.jo[n] = 0.000000001;
  hd->grain_tot = 1;
  cudaMemcpyAsync(c->dev, hd, sizeof(hc_dev), cudaMemcpyHostToDevice, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    free_all(c);
    return HC_ERR_CUDA;
  }
  *out = c;
  return HC_OK;
}

static hc_status free_all(hc_ctx* c) {
  hc_view& v = c->v;
  void* ptrs[] = {v.elev, v.h, v.qx, v.qy, v.qxs, v.qys, v.vs, v.vel, v.tau, v.bed, v.man,
                  v.area, v.ss, v.vd, v.sflux, v.grain, v.strata, v.index, v.mask, v.rfarea,
                  v.edge, v.edge2, v.veg, v.cin_x, v.cin_y, v.erodetot, v.erodetot3, v.pre,
                  v.chains, v.ent_list, v.ent_qs, v.drain_pos, v.drain_f0, v.drain_f1, v.drain_pend, v.drain_dt, v.drain_frac, v.drain_multi,
                  v.drain_snap, v.drain_aux, v.alloc_key, v.red, v.touched, v.topm, v.rain, v.rec, c->dev, v.wet,
                  v.wet_sums, v.vpart, v.sdirty, v.border,
                  v.reach[0], v.reach[1], v.reach[2], extra(c).lateral};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (c->hdev) cudaFreeHost(c->hdev);
  if (c->h_elev) cudaFreeHost(c->h_elev);
  if (c->drainage_cache) host_drainage_cache_free(c->drainage_cache);
  sort_work_free(c->sort_work);
  free(extra(c).h_rain);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  for (auto& t : c->tail)
    if (t) cudaGraphExecDestroy(t);
  if (c->chunk_done) cudaEventDestroy(c->chunk_done);
  if (c->s) cudaStreamDestroy(c->s);
  if (c->s2) cudaStreamDestroy(c->s2);
  if (c->s3) cudaStreamDestroy(c->s3);
  drop_extra(c);
  delete c;
  return HC_OK;
}

extern "C" hc_status hc_destroy(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  cudaStreamSynchronize(c->s);
  return free_all(c);
}

// ------------------------------------------------------------------ transfers
static double* plain_field(hc_ctx* c, hc_field f) {
  hc_view& v = c->v;
  switch (f) {
    case HC_F_ELEV: return v.elev;
    case HC_F_WATER_DEPTH: return v.h;
    case HC_F_QX: return v.qx;
    case HC_F_QY: return v.qy;
    case HC_F_QXS: return v.qxs;
    case HC_F_QYS: return v.qys;
    case HC_F_VSUSPTOT: return v.vs;
    case HC_F_VEL: return v.vel;
    case HC_F_TAU: return v.tau;
    case HC_F_BEDROCK: return v.bed;
    case HC_F_MANNINGS: return v.man;
    case HC_F_AREA: return v.area;
    case HC_F_SS: return v.ss;
    case HC_F_EDGE: return v.edge;
    case HC_F_VEG: return v.veg;
    default: return nullptr;
  }
}

static int sflux_dir(hc_field f) {
  switch (f) {
    case HC_F_SU: return 0;
    case HC_F_SR: return 1;
    case HC_F_SD: return 2;
    case HC_F_SL: return 3;
    default: return -1;
  }
}

static hc_status check_size(hc_ctx* c, hc_field f, size_t nbytes) {
  const int64_t n = hc_field_count(&c->v.p, f);
  const int32_t es = hc_field_elsize(f);
  if (n < 0 || es < 0) return hc_fail(c, HC_ERR_ARG, "unknown field %d", (int)f);
  if ((size_t)n * es != nbytes)
    return hc_fail(c, HC_ERR_ARG, "field %d: %zu bytes given, %lld expected", (int)f, nbytes,
                   (long long)n * es);
  if (c->v.p.hydro_only && (f == HC_F_GRAIN || f == HC_F_STRATA || sflux_dir(f) >= 0))
    return hc_fail(c, HC_ERR_STATE, "field %d is not kept in hydro-only mode", (int)f);
  return HC_OK;
}

extern "C" hc_status hc_upload(hc_ctx* c, hc_field f, const void* host, size_t nbytes) {
  if (!c || !host) return HC_ERR_ARG;
  HC_TRY(check_size(c, f, nbytes));
  c->h2d_bytes += nbytes;
  hc_view& v = c->v;
  const size_t N2 = v.N2;
  cudaStream_t s = c->s;
  if (double* d = plain_field(c, f)) {
    HC_CU(cudaMemcpyAsync(d, host, nbytes, cudaMemcpyHostToDevice, s), "upload");
    HC_CU(cudaStreamSynchronize(s), "upload");
    if (f == HC_F_ELEV || f == HC_F_AREA) c->area_valid = false;
    if (f == HC_F_ELEV && c->drainage_cache) {  // the cached elevation order is stale
      host_drainage_cache_free(c->drainage_cache);
      c->drainage_cache = nullptr;
    }
    return HC_OK;
  }
  switch (f) {
    case HC_F_INDEX:
      HC_CU(cudaMemcpyAsync(v.index, host, nbytes, cudaMemcpyHostToDevice, s), "upload");
      break;
    case HC_F_RFAREA:
      HC_CU(cudaMemcpyAsync(v.rfarea, host, nbytes, cudaMemcpyHostToDevice, s), "upload");
      break;
    case HC_F_INPUTPOINTS:
      // The reference clears inputpointsarray in zero_values after marking
      // the reach cells (:2905), so the mask never affects a run; accepted
      // and ignored.
      break;
    case HC_F_VEL_DIR: {
      std::vector<double> planes(4 * N2);
      const double* h = (const double*)host;
      for (size_t cell = 0; cell < N2; cell++)
        for (int k = 0; k < 4; k++) planes[(size_t)k * N2 + cell] = h[cell * 9 + 1 + 2 * k];
      HC_CU(cudaMemcpy(v.vd, planes.data(), 4 * N2 * 8, cudaMemcpyHostToDevice), "upload");
      break;
    }
    case HC_F_SR: case HC_F_SL: case HC_F_SU: case HC_F_SD: {
      const int dir = sflux_dir(f);
      std::vector<double> planes(10 * N2);
      const double* h = (const double*)host;
      for (size_t cell = 0; cell < N2; cell++)
        for (int n = 0; n < 10; n++) planes[(size_t)n * N2 + cell] = h[cell * 10 + n];
      HC_CU(cudaMemcpy(v.sflux + (size_t)dir * 10 * N2, planes.data(), 10 * N2 * 8,
                       cudaMemcpyHostToDevice), "upload");
      HC_CU(cudaMemset(v.sdirty, 1, N2), "upload");  // any entry may be nonzero now
      break;
    }
    case HC_F_GRAIN: case HC_F_STRATA: {
      // rows addressed by index[][]: scatter into the cells' slots
      std::vector<int32_t> idx(N2);
      HC_CU(cudaMemcpy(idx.data(), v.index, N2 * 4, cudaMemcpyDeviceToHost), "upload");
      const int64_t nrec = (int64_t)N2 / std::max(1, v.p.LIMIT);
      const double* h = (const double*)host;
      if (f == HC_F_GRAIN) {
        std::vector<double> slots(kGrainStride * N2, 0.0);
        for (size_t cell = 0; cell < N2; cell++) {
          const int r = idx[cell];
          if (r < 0 || r >= nrec) continue;
          for (int n = 0; n < 11; n++) slots[cell * kGrainStride + n] = h[(size_t)r * 11 + n];
        }
        HC_CU(cudaMemcpy(v.grain, slots.data(), slots.size() * 8, cudaMemcpyHostToDevice),
              "upload");
      } else {
        std::vector<double> slots(kStrataStride * N2, 0.0);
        for (size_t cell = 0; cell < N2; cell++) {
          const int r = idx[cell];
          if (r < 0 || r >= nrec) continue;
          for (int z = 0; z < 10; z++)
            for (int n = 0; n < 9; n++)
              slots[cell * kStrataStride + (size_t)z * 9 + n] = h[((size_t)r * 10 + z) * 11 + n];
        }
        HC_CU(cudaMemcpy(v.strata, slots.data(), slots.size() * 8, cudaMemcpyHostToDevice),
              "upload");
      }
      break;
    }
    case HC_F_DOWN_SCAN: {
      // lists of wet rows per column -> per-cell mask
      const int32_t* ds = (const int32_t*)host;
      std::vector<uint8_t> m(N2, 0);
      const int I = v.imax, J = v.jmax;
      for (int j = 1; j <= J; j++) {
        int k = 1;
        while (k <= I + 1 && ds[(size_t)j * (I + 2) + k] > 0) {
          int i = ds[(size_t)j * (I + 2) + k];
          if (i >= 1 && i <= I) m[(size_t)i * v.W + j] = 1;
          k++;
        }
      }
      HC_CU(cudaMemcpy(v.mask, m.data(), N2, cudaMemcpyHostToDevice), "upload");
      launch_wet_list(c, 0);
      break;
    }
    default:
      return hc_fail(c, HC_ERR_ARG, "field %d cannot be uploaded", (int)f);
  }
  HC_CU(cudaStreamSynchronize(s), "upload");
  return HC_OK;
}

extern "C" hc_status hc_download(hc_ctx* c, hc_field f, void* host, size_t nbytes) {
  if (!c || !host) return HC_ERR_ARG;
  HC_TRY(check_size(c, f, nbytes));
  c->d2h_bytes += nbytes;
  hc_view& v = c->v;
  const size_t N2 = v.N2;
  cudaStream_t s = c->s;
  HC_CU(cudaStreamSynchronize(s), "download");
  if (double* d = plain_field(c, f)) {
    HC_CU(cudaMemcpy(host, d, nbytes, cudaMemcpyDeviceToHost), "download");
    return HC_OK;
  }
  switch (f) {
    case HC_F_INDEX:
      HC_CU(cudaMemcpy(host, v.index, nbytes, cudaMemcpyDeviceToHost), "download");
      break;
    case HC_F_RFAREA:
      HC_CU(cudaMemcpy(host, v.rfarea, nbytes, cudaMemcpyDeviceToHost), "download");
      break;
    case HC_F_INPUTPOINTS:
      std::memset(host, 0, nbytes);
      break;
    case HC_F_VEL_DIR: {
      std::vector<double> planes(4 * N2);
      HC_CU(cudaMemcpy(planes.data(), v.vd, 4 * N2 * 8, cudaMemcpyDeviceToHost), "download");
      double* h = (double*)host;
      std::memset(h, 0, nbytes);
      for (size_t cell = 0; cell < N2; cell++)
        for (int k = 0; k < 4; k++) h[cell * 9 + 1 + 2 * k] = planes[(size_t)k * N2 + cell];
      break;
    }
    case HC_F_SR: case HC_F_SL: case HC_F_SU: case HC_F_SD: {
      const int dir = sflux_dir(f);
      std::vector<double> planes(10 * N2);
      HC_CU(cudaMemcpy(planes.data(), v.sflux + (size_t)dir * 10 * N2, 10 * N2 * 8,
                       cudaMemcpyDeviceToHost), "download");
      double* h = (double*)host;
      for (size_t cell = 0; cell < N2; cell++)
        for (int n = 0; n < 10; n++) h[cell * 10 + n] = planes[(size_t)n * N2 + cell];
      break;
    }
    case HC_F_GRAIN: case HC_F_STRATA: {
      std::vector<int32_t> idx(N2);
      HC_CU(cudaMemcpy(idx.data(), v.index, N2 * 4, cudaMemcpyDeviceToHost), "download");
      const int64_t nrec = (int64_t)N2 / std::max(1, v.p.LIMIT);
      double* h = (double*)host;
      std::memset(h, 0, nbytes);
      if (f == HC_F_GRAIN) {
        std::vector<double> slots(kGrainStride * N2);
        HC_CU(cudaMemcpy(slots.data(), v.grain, slots.size() * 8, cudaMemcpyDeviceToHost),
              "download");
        for (size_t cell = 0; cell < N2; cell++) {
          const int r = idx[cell];
          if (r < 0 || r >= nrec) continue;
          for (int n = 0; n < 11; n++) h[(size_t)r * 11 + n] = slots[cell * kGrainStride + n];
        }
      } else {
        std::vector<double> slots(kStrataStride * N2);
        HC_CU(cudaMemcpy(slots.data(), v.strata, slots.size() * 8, cudaMemcpyDeviceToHost),
              "download");
        for (size_t cell = 0; cell < N2; cell++) {
          const int r = idx[cell];
          if (r < 0 || r >= nrec) continue;
          for (int z = 0; z < 10; z++)
            for (int n = 0; n < 9; n++)
              h[((size_t)r * 10 + z) * 11 + n] = slots[cell * kStrataStride + (size_t)z * 9 + n];
        }
      }
      break;
    }
    case HC_F_DOWN_SCAN: {
      std::vector<uint8_t> m(N2);
      HC_CU(cudaMemcpy(m.data(), v.mask, N2, cudaMemcpyDeviceToHost), "download");
      int32_t* ds = (int32_t*)host;
      std::memset(ds, 0, nbytes);
      const int I = v.imax, J = v.jmax;
      for (int j = 1; j <= J; j++) {
        int k = 1;
        for (int i = 1; i <= I; i++)
          if (m[(size_t)i * v.W + j]) ds[(size_t)j * (I + 2) + (k++)] = i;
      }
      break;
    }
    default:
      return hc_fail(c, HC_ERR_ARG, "field %d cannot be downloaded", (int)f);
  }
  return HC_OK;
}

// ------------------------------------------------------------------ snapshots
// A field's copy taken in stream order (a device-to-device copy, so the run
// can go on at once) and moved to pinned host memory on a side stream.
struct hc_snapshot {
  hc_ctx* c;
  double* dev;
  cudaEvent_t taken, done;
};

extern "C" hc_status hc_snapshot_begin(hc_ctx* c, hc_field f, void* host_pinned, size_t nbytes,
                                       hc_snapshot** out) {
  if (!c || !host_pinned || !out) return HC_ERR_ARG;
  *out = nullptr;
  double* src = plain_field(c, f);
  if (!src) return hc_fail(c, HC_ERR_ARG, "field %d has no plain layout for a snapshot", (int)f);
  HC_TRY(check_size(c, f, nbytes));
  hc_snapshot* sn = new hc_snapshot();
  sn->c = c;
  if (cudaMalloc((void**)&sn->dev, nbytes) != cudaSuccess) {
    cudaGetLastError();
    delete sn;
    return hc_fail(c, HC_ERR_NOMEM, "snapshot buffer");
  }
  cudaEventCreateWithFlags(&sn->taken, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&sn->done, cudaEventDisableTiming);
  HC_CU(cudaMemcpyAsync(sn->dev, src, nbytes, cudaMemcpyDeviceToDevice, c->s), "snapshot");
  if (!c->s3) HC_CU(cudaStreamCreateWithFlags(&c->s3, cudaStreamNonBlocking), "snapshot stream");
  HC_CU(cudaEventRecord(sn->taken, c->s), "snapshot");
  HC_CU(cudaStreamWaitEvent(c->s3, sn->taken, 0), "snapshot");
  HC_CU(cudaMemcpyAsync(host_pinned, sn->dev, nbytes, cudaMemcpyDeviceToHost, c->s3), "snapshot");
  HC_CU(cudaEventRecord(sn->done, c->s3), "snapshot");
  c->d2h_bytes += nbytes;
  *out = sn;
  return HC_OK;
}

extern "C" hc_status hc_snapshot_end(hc_snapshot* sn) {
  if (!sn) return HC_ERR_ARG;
  hc_ctx* c = sn->c;
  const cudaError_t e = cudaEventSynchronize(sn->done);
  cudaEventDestroy(sn->taken);
  cudaEventDestroy(sn->done);
  cudaFree(sn->dev);
  delete sn;
  return hc_cuda(c, e, "snapshot");
}

// ------------------------------------------------------------------ series
extern "C" hc_status hc_set_rain(hc_ctx* c, const float* rain, int32_t rows, int32_t cols) {
  if (!c || !rain || rows <= 0 || cols <= 0) return HC_ERR_ARG;
  Extra& x = extra(c);
  free(x.h_rain);
  x.h_rain = (float*)malloc((size_t)rows * cols * 4);
  std::memcpy(x.h_rain, rain, (size_t)rows * cols * 4);
  x.h_rain_rows = rows;
  x.h_rain_cols = cols;
  hc_view& v = c->v;
  if (v.rain) cudaFree(v.rain);
  v.rain = nullptr;
  HC_TRY(dalloc(c, &v.rain, (size_t)rows * cols));
  HC_CU(cudaMemcpy(v.rain, rain, (size_t)rows * cols * 4, cudaMemcpyHostToDevice), "rain");
  v.rain_rows = rows;
  v.rain_cols = cols;
  c->prepared = false;
  return HC_OK;
}

extern "C" hc_status hc_set_reach(hc_ctx* c, int32_t point, const float* data, int32_t rows,
                                  int32_t cols) {
  if (!c || !data || point < 0 || point >= HC_MAX_POINTS || rows <= 0 || cols < 14)
    return HC_ERR_ARG;
  hc_view& v = c->v;
  if (v.reach[point]) cudaFree(v.reach[point]);
  v.reach[point] = nullptr;
  HC_TRY(dalloc(c, &v.reach[point], (size_t)rows * cols));
  HC_CU(cudaMemcpy(v.reach[point], data, (size_t)rows * cols * 4, cudaMemcpyHostToDevice), "reach");
  v.reach_rows[point] = rows;
  v.reach_cols[point] = cols;
  c->graph_iters = 0;
  return HC_OK;
}

// ------------------------------------------------------------------ scalars
// a device-side error (HC_PAUSE_ERROR) as a status
static hc_status device_error(hc_ctx* c) {
  const int e = c->hdev->err_code;
  if (e == 301) return hc_fail(c, HC_ERR_NONFINITE, "non-finite water depth (device error 301)");
  if (e == 401) return hc_fail(c, HC_ERR_TIMEOUT, "drainage sweep: a device wait gave up (401)");
  return hc_fail(c, HC_ERR_STATE, "device error %d", e);
}

static hc_status pull(hc_ctx* c) {
  c->d2h_bytes += sizeof(hc_dev);
  HC_CU(cudaMemcpyAsync(c->hdev, c->dev, sizeof(hc_dev), cudaMemcpyDeviceToHost, c->s), "pull");
  HC_CU(cudaStreamSynchronize(c->s), "pull");
  return HC_OK;
}
static hc_status push(hc_ctx* c) {
  c->h2d_bytes += sizeof(hc_dev);
  HC_CU(cudaMemcpyAsync(c->dev, c->hdev, sizeof(hc_dev), cudaMemcpyHostToDevice, c->s), "push");
  HC_CU(cudaStreamSynchronize(c->s), "push");
  return HC_OK;
}

// for the other translation units of the library
hc_status ctx_pull(hc_ctx* c) { return pull(c); }
hc_status ctx_push(hc_ctx* c) { return push(c); }
const float* ctx_rain(hc_ctx* c, int* rows, int* cols) {
  Extra& x = extra(c);
  *rows = x.h_rain_rows;
  *cols = x.h_rain_cols;
  return x.h_rain;
}

extern "C" hc_status hc_get_scalars(hc_ctx* c, hc_scalars* s) {
  if (!c || !s) return HC_ERR_ARG;
  HC_TRY(pull(c));
  c->hdev->s.grain_array_tot = c->hdev->grain_tot;
  *s = c->hdev->s;
  return HC_OK;
}

extern "C" hc_status hc_set_scalars(hc_ctx* c, const hc_scalars* s) {
  if (!c || !s) return HC_ERR_ARG;
  HC_TRY(pull(c));
  c->hdev->s = *s;
  c->hdev->grain_tot = (int)s->grain_array_tot;
  return push(c);
}

// ------------------------------------------------------------------ prepare
// accumulates the host wall time of a piece of hc_run's host work
namespace {
struct StatTimer {
  hc_ctx* c;
  int k;
  std::chrono::steady_clock::time_point t0;
  StatTimer(hc_ctx* c_, int k_) : c(c_), k(k_), t0(std::chrono::steady_clock::now()) {}
  ~StatTimer() {
    c->stat_n[k]++;
    c->stat_ms[k] +=
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
};
}  // namespace

// the drainage sweep order, sorted on the device; the host's exact sort
// when the device declines (depth budget exhausted, NaN elevations)
static hc_status drainage_sort(hc_ctx* c, const double* del, uint32_t* order_dev) {
  StatTimer st(c, HC_STAT_DRAINAGE_SORT);
  bool fallback = false;
  HC_CU(device_drainage_order(c, del, order_dev, &fallback), "drainage sort");
  if (!fallback) return HC_OK;
  StatTimer hs(c, HC_STAT_DRAINAGE_HOST_SORT);
  const size_t N2 = c->v.N2;
  std::vector<double> elev(N2);
  HC_CU(cudaMemcpy(elev.data(), del, N2 * 8, cudaMemcpyDeviceToHost), "drainage sort");
  c->d2h_bytes += N2 * 8;
  if (!c->drainage_cache) c->drainage_cache = host_drainage_cache_new();
  bool reused = false;
  const uint32_t* order = host_drainage_order(&c->v.p, elev.data(), c->drainage_cache, &reused);
  HC_CU(cudaMemcpy(order_dev, order, N2 * 4, cudaMemcpyHostToDevice), "drainage sort");
  c->h2d_bytes += N2 * 4;
  return HC_OK;
}

// zero_and_calc_drainage_area + get_catchment_input_points (hc_drain.cu).
// `snapshot`: use the elevations copied at the start of the iteration that
// moved the baseflow threshold (erosion has changed elev since).  Hydro-only
// runs never change elevations, so their area is computed once.
static hc_status recompute_points(hc_ctx* c, bool snapshot) {
  hc_view& v = c->v;
  const double* del = (snapshot && v.drain_snap) ? v.drain_snap : v.elev;
  HC_TRY(push(c));  // baseflow
  bool sorted = false;
  const bool keep_area = c->area_valid && v.p.hydro_only;
  if (run_drainage_device(c, del, keep_area, drainage_sort, &sorted) != HC_OK)
    return hc_cuda(c, cudaGetLastError(), "drainage");
  HC_CU(cudaStreamSynchronize(c->s), "drainage");
  c->area_valid = true;
  HC_TRY(pull(c));
  if ((c->hdev->pause & HC_PAUSE_ERROR) && c->hdev->err_code == 401) {
    // a bounded wait of the sweep ran out: the context stays usable, and
    // the next hc_run makes this recomputation again before its iterations
    const hc_status st = device_error(c);
    c->hdev->err_code = 0;
    c->hdev->pause &= ~HC_PAUSE_ERROR;
    c->area_valid = false;
    c->drain_retry = true;
    HC_TRY(push(c));
    return st;
  }
  if (c->hdev->pause & HC_PAUSE_ERROR) return device_error(c);
  c->drain_retry = false;
  if (!keep_area) c->stat_n[HC_STAT_DRAINAGE_LEVELS] += c->hdev->drain_levels;
  if (c->points_hook) c->points_hook(c, c->points_hook_arg);
  return HC_OK;
}

extern "C" hc_status hc_prepare(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  hc_view& v = c->v;
  const hc_params& p = v.p;
  Extra& x = extra(c);
  if (!x.h_rain) return hc_fail(c, HC_ERR_STATE, "hc_set_rain must come before hc_prepare");
  for (int n = 0; n < p.number_of_points && p.reach_mode; n++)
    if (!v.reach[n]) return hc_fail(c, HC_ERR_STATE, "reach table %d missing", n);
  const size_t N2 = v.N2;
  std::vector<double> elev(N2);
  std::vector<int32_t> rf(N2);
  HC_CU(cudaStreamSynchronize(c->s), "prepare");
  HC_CU(cudaMemcpy(elev.data(), v.elev, N2 * 8, cudaMemcpyDeviceToHost), "prepare");
  HC_CU(cudaMemcpy(rf.data(), v.rfarea, N2 * 4, cudaMemcpyDeviceToHost), "prepare");
  HC_TRY(pull(c));
  hc_scalars& s = c->hdev->s;
  for (int n = 0; n <= HC_MAX_RF; n++) s.nActualGridCells[n] = 0;
  for (int i = 1; i < p.imax; i++)  // count_catchment_gridcells :2813 (i < imax, j < jmax)
    for (int j = 1; j < p.jmax; j++)
      if (elev[(size_t)i * v.W + j] > -9999) {
        const int r = rf[(size_t)i * v.W + j];
        if (r < 0 || r > p.rfnum) return hc_fail(c, HC_ERR_ARG, "rfarea value %d out of range", r);
        s.nActualGridCells[r] += 1;
      }
  s.creep_time = s.creep_time2 = s.time_1 = s.cycle;  // set_time_counters :1862
  // TOPMODEL rows: initialise_rainfall_runoff's call, then one per minute
  const int rows = p.maxcycle * 60 + std::max(0, p.max_time_step / 60) + 2000;
  std::vector<double> table((size_t)rows * 2 * (p.rfnum + 1));
  host_topmodel_table(&p, x.h_rain, x.h_rain_rows, x.h_rain_cols, rows, table.data());
  if (v.topm) cudaFree(v.topm);
  v.topm = nullptr;
  HC_TRY(dalloc(c, &v.topm, table.size()));
  HC_CU(cudaMemcpy(v.topm, table.data(), table.size() * 8, cudaMemcpyHostToDevice), "prepare");
  v.topm_rows = rows;
  for (int n = p.spatially_complex_rainfall ? 0 : 1; n <= p.rfnum; n++) {
    s.old_j_mean[n] = table[n];
    s.new_j_mean[n] = table[(p.rfnum + 1) + n];
  }
  for (int n = 1; n <= 9; n++) v.dlog[n] = std::log(p.d[n]);
  if (p.spatially_complex_rainfall) {
    // distributed runoff: the computed cells (rows 1 .. imax-1, columns
    // 1 .. jmax-1, above no-data) per rain state; initialise_drainage_area
    // skips the drainage area and the input points in this mode (:2055-2070)
    for (int z = 0; z <= HC_MAX_RF; z++) v.runoff_count[z] = 0;
    v.runoff_present = 0;
    for (int i = 1; i < p.imax; i++)
      for (int j = 1; j < p.jmax; j++) {
        const size_t cell = (size_t)i * v.W + j;
        if (!(elev[cell] > -9999)) continue;
        const int r = rf[cell];
        const int z = (p.rfnum == 1) ? 1 : ((r >= 1 && r <= p.rfnum - 1) ? r : 0);
        v.runoff_count[z] += 1;
        v.runoff_present |= 1u << z;
      }
    HC_TRY(push(c));
  } else {
    HC_TRY(push(c));
    HC_TRY(recompute_points(c, false));
  }
  c->prepared = true;
  c->graph_iters = 0;  // parameters of the view changed: rebuild the graph
  launch_mass_reset(c);  // the water ledger starts from the state as prepared
  HC_TRY(pull(c));
  return HC_OK;
}

// ------------------------------------------------------------------ water ledger
extern "C" hc_status hc_mass_balance(hc_ctx* c, hc_mass* m) {
  if (!c || !m) return HC_ERR_ARG;
  launch_volume(c);
  HC_TRY(pull(c));
  const hc_dev* d = c->hdev;
  const double a2 = c->v.p.DX * c->v.p.DX;
  m->volume0 = d->vol0 * a2;
  m->volume = d->vol_now * a2;
  // terms of an iteration whose water_flux_out has not run yet count too
  m->inflow = (d->vin_tot + d->vin_step) * a2;
  m->outflow = d->vout_tot * a2;
  m->lost = (d->vlost_tot + d->vlost_step) * a2;
  m->mask_edge = (d->vmask_tot + d->vmask_step) * a2;
  return HC_OK;
}

extern "C" hc_status hc_mass_reset(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  launch_mass_reset(c);
  return pull(c);
}

// ------------------------------------------------------------------ members
extern "C" hc_status hc_set_maximum_timestep(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  k_set_max_ts<<<1, 1, 0, c->s>>>(c->v, c->dev);
  HC_CU(cudaStreamSynchronize(c->s), "set_maximum_timestep");
  return HC_OK;
}

extern "C" hc_status hc_flow_route(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  launch_flow_dt(c);
  launch_flow_route(c, 0);
  HC_CU(cudaStreamSynchronize(c->s), "flow_route");
  return HC_OK;
}

extern "C" hc_status hc_depth_update(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  launch_flow_dt(c);
  launch_depth_update(c, 0);
  HC_TRY(pull(c));
  if (c->hdev->pause & HC_PAUSE_ERROR) return device_error(c);
  return HC_OK;
}

extern "C" hc_status hc_scan_area(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  launch_scan_area(c, 0);
  HC_CU(cudaStreamSynchronize(c->s), "scan_area");
  return HC_OK;
}

extern "C" hc_status hc_water_flux_out(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  launch_flux_out(c, 0, 0);
  HC_CU(cudaStreamSynchronize(c->s), "water_flux_out");
  return HC_OK;
}

extern "C" hc_status hc_erode(hc_ctx* c, double mult, double* tempbmax) {
  if (!c) return HC_ERR_ARG;
  if (c->v.p.hydro_only) return hc_fail(c, HC_ERR_STATE, "erosion arrays absent (hydro_only)");
  if (!c->prepared) {
    for (int n = 1; n <= 9; n++) c->v.dlog[n] = std::log(c->v.p.d[n]);
  }
  launch_erode_begin(c, 0, mult < 0 ? 0 : mult);
  for (int guard = 0;; guard++) {
    launch_erode_pass(c, 0);
    HC_TRY(pull(c));
    if (c->hdev->pause & HC_PAUSE_ERROR)
      return device_error(c);
    if (!c->hdev->erode_retry) break;
    if (guard > 100000) return hc_fail(c, HC_ERR_TIMEOUT, "erosion retry loop did not end");
  }
  launch_erode_finish(c, 0);
  HC_TRY(pull(c));
  if (tempbmax) *tempbmax = c->hdev->s.tempbmax;
  return HC_OK;
}

extern "C" hc_status hc_lateral_channel_erode(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  if (c->v.p.hydro_only) return hc_fail(c, HC_ERR_STATE, "erosion arrays absent (hydro_only)");
  return run_lateral(c);
}

extern "C" hc_status hc_in_channel_landsliding(hc_ctx* c) {
  if (!c) return HC_ERR_ARG;
  if (c->v.p.hydro_only) return hc_fail(c, HC_ERR_STATE, "erosion arrays absent (hydro_only)");
  launch_slide3(c, 0);
  HC_TRY(pull(c));
  if (c->hdev->pause & HC_PAUSE_ERROR)
    return device_error(c);
  return HC_OK;
}

extern "C" hc_status hc_global_landsliding(hc_ctx* c, int32_t* sweeps) {
  if (!c) return HC_ERR_ARG;
  if (c->v.p.hydro_only) return hc_fail(c, HC_ERR_STATE, "erosion arrays absent (hydro_only)");
  int n = 0;
  HC_TRY(run_global_landsliding(c, &n));
  if (sweeps) *sweeps = n;
  HC_CU(cudaStreamSynchronize(c->s), "global_landsliding");
  return HC_OK;
}

extern "C" hc_status hc_creep(hc_ctx* c, double time) {
  if (!c) return HC_ERR_ARG;
  if (c->v.p.hydro_only) return hc_fail(c, HC_ERR_STATE, "erosion arrays absent (hydro_only)");
  HC_TRY(run_creep(c, time));
  HC_TRY(pull(c));
  if (c->hdev->pause & HC_PAUSE_ERROR) return device_error(c);
  return HC_OK;
}

// ------------------------------------------------------------------ hc_run
static void launch_iteration(hc_ctx* c, int flags) {
  launch_control(c);
  launch_inputs(c);
  launch_flow_route(c, 1);
  launch_depth_update(c, 1);
  launch_scan_area(c, 1);
  if (!c->v.p.hydro_only) {
    for (int k = 0; k < HC_ERODE_PASSES; k++) launch_erode_pass(c, HC_ERODE_PASSES);
    launch_erode_finish(c, 1);
    if (flags & HC_RUN_LATERAL) launch_lateral_check(c);
  }
  launch_flux_out(c, 1, 1);
  if (!c->v.p.hydro_only) launch_slide3(c, 1);
}

// Adds an IF node at the current capture position of c->s whose body is
// captured from the launches `fn` issues (on the side stream).
template <class F>
static hc_status capture_if(hc_ctx* c, cudaGraphConditionalHandle h, F fn) {
  cudaStreamCaptureStatus st;
  cudaGraph_t cg;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  HC_CU(cudaStreamGetCaptureInfo(c->s, &st, nullptr, &cg, &deps, nullptr, &nd), "capture info");
  cudaGraphNodeParams prm = {};
  prm.type = cudaGraphNodeTypeConditional;
  prm.conditional.handle = h;
  prm.conditional.type = cudaGraphCondTypeIf;
  prm.conditional.size = 1;
  cudaGraphNode_t node;
  HC_CU(cudaGraphAddNode(&node, cg, deps, nullptr, nd, &prm), "conditional node");
  cudaGraph_t body = prm.conditional.phGraph_out[0];
  HC_CU(cudaStreamBeginCaptureToGraph(c->s2, body, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed), "body capture");
  c->cs = c->s2;
  fn();
  c->cs = c->s;
  cudaGraph_t out;
  HC_CU(cudaStreamEndCapture(c->s2, &out), "body capture");
  HC_CU(cudaStreamUpdateCaptureDependencies(c->s, &node, nullptr, 1,
                                            cudaStreamSetCaptureDependencies), "dependencies");
  return HC_OK;
}

// One iteration as captured into the graph: the same launches as
// launch_iteration, with the steps that are not due every iteration behind
// IF nodes (scan_area, the erosion block and its extra passes, slide_3).
static hc_status capture_iteration(hc_ctx* c, int flags) {
  cudaStreamCaptureStatus st;
  cudaGraph_t cg;
  HC_CU(cudaStreamGetCaptureInfo(c->s, &st, nullptr, &cg, nullptr, nullptr, nullptr), "capture info");
  hc_iter_handles& H = c->hcur;
  std::memset(&H, 0, sizeof H);
  const bool sed = !c->v.p.hydro_only;
  auto mk = [&](cudaGraphConditionalHandle* h) {
    return cudaGraphConditionalHandleCreate(h, cg, 0, cudaGraphCondAssignDefault);
  };
  HC_CU(mk(&H.scan), "handle");
  if (sed) {
    HC_CU(mk(&H.erode), "handle");
    HC_CU(mk(&H.retry2), "handle");
    HC_CU(mk(&H.retry3), "handle");
    HC_CU(mk(&H.retry4), "handle");
    HC_CU(mk(&H.erode_fin), "handle");
    HC_CU(mk(&H.slide), "handle");
  }
  H.has = 1;
  launch_control(c);
  H.has = 0;  // no other launch sets the iteration's conditions
  if (c->v.adj_sh) launch_adj_save(c);
  launch_inputs(c);
  launch_flow_route(c, 1);
  launch_depth_update(c, 1);
  HC_TRY(capture_if(c, H.scan, [&] { launch_scan_area(c, 1); }));
  if (sed) {
    const hc_iter_handles h = H;
    HC_TRY(capture_if(c, h.erode, [&] { launch_erode_pass(c, HC_ERODE_PASSES, h.retry2, 1); }));
    HC_TRY(capture_if(c, h.retry2, [&] { launch_erode_pass(c, HC_ERODE_PASSES, h.retry3, 1); }));
    HC_TRY(capture_if(c, h.retry3, [&] { launch_erode_pass(c, HC_ERODE_PASSES, h.retry4, 1); }));
    HC_TRY(capture_if(c, h.retry4, [&] { launch_erode_pass(c, HC_ERODE_PASSES); }));
    HC_TRY(capture_if(c, h.erode_fin, [&] { launch_erode_finish(c, 1); }));
    if (flags & HC_RUN_LATERAL) launch_lateral_check(c);
    launch_flux_out(c, 1, 1);
    HC_TRY(capture_if(c, h.slide, [&] { launch_slide3(c, 1); }));
  } else {
    launch_flux_out(c, 1, 1);
  }
  return HC_OK;
}

// iterations per chunk graph: HC_GRAPH_ITERS if set, else what the caller
// asked for (hc_run_ensemble: 128), else 32
static int graph_chunk(const hc_ctx* c) {
  const char* e = getenv("HC_GRAPH_ITERS");
  int k = e ? atoi(e) : (c->chunk_pref > 0 ? c->chunk_pref : 32);
  return std::max(1, std::min(k, 4096));
}

// Captures K iterations into *exec; *kernels = kernel nodes outside
// conditional bodies (they run on every launch; those inside run only when
// their condition is set, and the device counts them).
static hc_status build_one(hc_ctx* c, int flags, int K, cudaGraphExec_t* exec,
                           int64_t* kernels) {
  if (*exec) cudaGraphExecDestroy(*exec);
  *exec = nullptr;
  cudaGraph_t g;
  HC_CU(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeRelaxed), "capture");
  c->capturing = true;
  hc_status cst = HC_OK;
  for (int k = 0; k < K && cst == HC_OK; k++) cst = capture_iteration(c, flags);
  c->capturing = false;
  c->cs = c->s;
  std::memset(&c->hcur, 0, sizeof c->hcur);
  cudaError_t ee = cudaStreamEndCapture(c->s, &g);
  if (cst != HC_OK) {
    if (ee == cudaSuccess) cudaGraphDestroy(g);
    return cst;
  }
  HC_CU(ee, "capture");
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  std::vector<cudaGraphNode_t> nodes(nn);
  cudaGraphGetNodes(g, nodes.data(), &nn);
  *kernels = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    cudaGraphNodeGetType(nd, &t);
    if (t == cudaGraphNodeTypeKernel) (*kernels)++;
  }
  cudaError_t e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  HC_CU(e, "graph instantiate");
  return HC_OK;
}

// The chunk graph (K iterations) and, for runs shorter than K, the graphs of
// 2^k < K iterations (a paused chunk skips the rest of its iterations, so a
// short run would otherwise pay for K).  All are made and uploaded here, so
// that no later hc_run instantiates a graph between its launches.
static hc_status build_graph(hc_ctx* c, int flags) {
  const int K = graph_chunk(c);
  for (auto& t : c->tail)
    if (t) {
      cudaGraphExecDestroy(t);
      t = nullptr;
    }
  HC_TRY(build_one(c, flags, K, &c->graph, &c->graph_kernels));
  HC_CU(cudaGraphUpload(c->graph, c->s), "graph upload");
  for (int k = 0; k < 12 && (1 << k) < K; k++) {
    HC_TRY(build_one(c, flags, 1 << k, &c->tail[k], &c->tail_kernels[k]));
    HC_CU(cudaGraphUpload(c->tail[k], c->s), "graph upload");
  }
  c->graph_iters = K;
  c->graph_flags = flags;
  return HC_OK;
}

// Finishes an iteration that stopped before water_flux_out (erosion retry
// beyond the captured passes, or lateral3 due).
static hc_status finish_iteration(hc_ctx* c, int flags) {
  hc_dev* hd = c->hdev;
  // the skipped iterations after the pause cleared it_active; this one resumes
  hd->it_active = 1;
  HC_TRY(push(c));
  if (hd->pause & HC_PAUSE_ERODE) {
    StatTimer st(c, HC_STAT_ERODE_RETRY);
    for (int guard = 0; hd->erode_retry; guard++) {
      launch_erode_pass(c, 0);
      HC_TRY(pull(c));
      if (guard > 100000) return hc_fail(c, HC_ERR_TIMEOUT, "erosion retry loop did not end");
    }
    hd->pause &= ~HC_PAUSE_ERODE;
    hd->rest_active = 1;
    HC_TRY(push(c));
    launch_erode_finish(c, 1);
    if (flags & HC_RUN_LATERAL) launch_lateral_check(c);
    HC_TRY(pull(c));
  }
  if (hd->pause & HC_PAUSE_LATERAL) {
    StatTimer st(c, HC_STAT_LATERAL);
    HC_TRY(run_lateral(c));
    HC_TRY(pull(c));
    hd->s.lateralcounter = hd->s.counter + (50 * hd->s.erode_mult);  // call_lateral :2302
    hd->do_lateral = 0;
    hd->pause &= ~HC_PAUSE_LATERAL;
    hd->rest_active = 1;
    HC_TRY(push(c));
  }
  launch_flux_out(c, 1, 1);
  if (!c->v.p.hydro_only) launch_slide3(c, 1);
  return pull(c);
}

static hc_status host_steps(hc_ctx* c, int flags) {
  hc_dev* hd = c->hdev;
  const hc_params& p = c->v.p;
  if (hd->pause & HC_PAUSE_HOSTSTEP) {
    hd->pause &= ~HC_PAUSE_HOSTSTEP;
    if (!p.hydro_only && !(flags & HC_RUN_NOHILL)) {
      if (hd->s.cycle > hd->s.creep_time) {  // slope_creep :1976
        StatTimer st(c, HC_STAT_CREEP);
        hd->s.creep_time += p.creep_time_interval;
        HC_TRY(push(c));
        HC_TRY(run_creep(c, p.creep_coeff));
        HC_TRY(pull(c));
      }
      if (hd->s.cycle > hd->s.creep_time2) {  // call_global_landsliding :1986
        StatTimer st(c, HC_STAT_GLOBAL_SLIDE);
        hd->s.creep_time2 += p.global_landsliding_interval;
        HC_TRY(push(c));
        HC_TRY(run_global_landsliding(c, nullptr));
        HC_TRY(pull(c));
      }
    }
    HC_TRY(push(c));
  }
  if (hd->pause & HC_PAUSE_DRAINAGE) {
    StatTimer st(c, HC_STAT_DRAINAGE);
    hd->pause &= ~HC_PAUSE_DRAINAGE;
    HC_TRY(push(c));
    HC_TRY(recompute_points(c, true));
  }
  return HC_OK;
}

// hc_run in pieces, so that hc_run_ensemble can keep several contexts' graphs
// in flight at once.
static hc_status run_begin(hc_ctx* c, int64_t n, int32_t flags, bool want_rec, bool* finished) {
  if (!c || n < 0) return HC_ERR_ARG;
  *finished = false;
  if (!c->prepared) return hc_fail(c, HC_ERR_STATE, "hc_prepare must come before hc_run");
  if ((flags & HC_RUN_LATERAL) && c->v.imax != c->v.jmax && !c->v.p.hydro_only)
    return hc_fail(c, HC_ERR_UNSUPPORTED, "lateral3 needs a square grid");
  hc_view& v = c->v;
  if (want_rec && v.rec_cap < n) {
    // at least 4096 records, so that short runs with records (one
    // iteration per call) do not rebuild the graphs as n grows
    const int64_t cap = std::max<int64_t>(n, 4096);
    if (v.rec) cudaFree(v.rec);
    v.rec = nullptr;
    v.rec_cap = 0;
    HC_TRY(dalloc(c, &v.rec, (size_t)cap));
    v.rec_cap = cap;
    c->graph_iters = 0;  // the view changed
  }
  HC_TRY(pull(c));
  hc_dev* hd = c->hdev;
  c->run_n = n;
  if (hd->pause & HC_PAUSE_FINISHED) {
    *finished = true;
    hd->budget = n;  // nothing runs
    return HC_OK;
  }
  hd->pause = 0;
  hd->budget = n;
  hd->rec_index = 0;
  hd->flags = flags;
  HC_TRY(push(c));
  if (c->drain_retry) {
    // the recomputation a timed-out wait left undone, from the elevations at
    // the start of the iteration that asked for it (erosion runs)
    StatTimer st(c, HC_STAT_DRAINAGE);
    HC_TRY(recompute_points(c, true));
    HC_TRY(pull(c));
  }
  HC_TRY(autotune(c, false));  // launch shapes for this shape class (hc_tune.cu)
  if (!c->graph_iters || c->graph_flags != flags || c->graph_iters != graph_chunk(c))
    HC_TRY(build_graph(c, flags));
  if (!c->chunk_done) HC_CU(cudaEventCreateWithFlags(&c->chunk_done, cudaEventDisableTiming),
                            "event");
  return HC_OK;
}

// one graph chunk, then the control block copied back; chunk_done marks both
static hc_status run_launch(hc_ctx* c) {
  c->body_k0 = c->hdev->body_kernels;
  c->budget0 = c->hdev->budget;
  c->stat_n[HC_STAT_CHUNKS]++;
  if (c->budget0 >= c->graph_iters) {
    c->chunk_iters = c->graph_iters;
    HC_CU(cudaGraphLaunch(c->graph, c->s), "graph launch");
    c->launches += c->graph_kernels;
  } else {
    int k = 0;
    while (k + 1 < 12 && (2LL << k) <= c->budget0) k++;
    if (!c->tail[k]) HC_TRY(build_one(c, c->graph_flags, 1 << k, &c->tail[k], &c->tail_kernels[k]));
    c->chunk_iters = 1 << k;
    HC_CU(cudaGraphLaunch(c->tail[k], c->s), "graph launch");
    c->launches += c->tail_kernels[k];
  }
  c->d2h_bytes += sizeof(hc_dev);
  HC_CU(cudaMemcpyAsync(c->hdev, c->dev, sizeof(hc_dev), cudaMemcpyDeviceToHost, c->s), "pull");
  HC_CU(cudaEventRecord(c->chunk_done, c->s), "event");
  return HC_OK;
}

// after a chunk: host-side work the device asked for; *finished when done
static hc_status run_after_chunk(hc_ctx* c, int32_t flags, bool* finished) {
  hc_dev* hd = c->hdev;
  *finished = false;
  c->launches += (int64_t)(hd->body_kernels - c->body_k0);
  c->stat_n[HC_STAT_IDLE_ITERS] += std::max<int64_t>(
      0, std::min<int64_t>(c->chunk_iters, c->budget0) - (c->budget0 - hd->budget));
  if (hd->pause & HC_PAUSE_ERROR) return device_error(c);
  if (hd->pause & (HC_PAUSE_ERODE | HC_PAUSE_LATERAL)) HC_TRY(finish_iteration(c, flags));
  HC_TRY(host_steps(c, flags));
  if ((hd->pause & HC_PAUSE_FINISHED) || hd->budget <= 0) {
    *finished = true;
    return HC_OK;
  }
  if (hd->pause & ~(HC_PAUSE_BUDGET)) {
    HC_TRY(pull(c));
    if (hd->pause & HC_PAUSE_ERROR)
      return device_error(c);
  }
  hd->pause &= HC_PAUSE_FINISHED;
  return push(c);
}

static hc_status run_end(hc_ctx* c, hc_step_record* rec, int64_t* done) {
  hc_dev* hd = c->hdev;
  const int64_t n = c->run_n;
  const int64_t ran = n - hd->budget;
  if (rec && ran > 0) {
    const int64_t nrec = std::min<int64_t>(hd->rec_index, n);
    c->d2h_bytes += nrec * (int64_t)sizeof(hc_step_record);
    HC_CU(cudaMemcpy(rec, c->v.rec, (size_t)nrec * sizeof(hc_step_record),
                     cudaMemcpyDeviceToHost), "records");
  }
  if (done) *done = ran;
  hd->pause &= HC_PAUSE_FINISHED;
  return push(c);
}

extern "C" hc_status hc_run(hc_ctx* c, int64_t n, int32_t flags, hc_step_record* rec,
                            int64_t* done) {
  if (done) *done = 0;
  bool finished = false;
  HC_TRY(run_begin(c, n, flags, rec != nullptr, &finished));
  while (!finished) {
    HC_TRY(run_launch(c));
    HC_CU(cudaEventSynchronize(c->chunk_done), "graph");
    HC_TRY(run_after_chunk(c, flags, &finished));
  }
  return run_end(c, rec, done);
}

// The service loop of a group of members: launch each member's first chunk,
// then, whichever member's chunk has finished, do its host work and launch
// its next chunk.
static hc_status ensemble_group(hc_ctx** ctxs, const std::vector<int>& mine, int64_t n,
                                int32_t flags, int64_t* done) {
  std::vector<char> live(mine.size(), 0);
  int left = 0;
  for (size_t q = 0; q < mine.size(); q++) {
    const int k = mine[q];
    bool fin = false;
    HC_TRY(run_begin(ctxs[k], n, flags, false, &fin));
    if (!fin) {
      HC_TRY(run_launch(ctxs[k]));
      live[q] = 1;
      left++;
    }
  }
  while (left > 0) {
    bool progressed = false;
    for (size_t q = 0; q < mine.size(); q++) {
      if (!live[q]) continue;
      const int k = mine[q];
      hc_ctx* c = ctxs[k];
      const cudaError_t e = cudaEventQuery(c->chunk_done);
      if (e == cudaErrorNotReady) continue;
      if (e != cudaSuccess) return hc_cuda(c, e, "ensemble");
      progressed = true;
      bool fin = false;
      HC_TRY(run_after_chunk(c, flags, &fin));
      if (fin) {
        HC_TRY(run_end(c, nullptr, done ? &done[k] : nullptr));
        live[q] = 0;
        left--;
      } else {
        HC_TRY(run_launch(c));
      }
    }
    if (!progressed) std::this_thread::yield();
  }
  return HC_OK;
}

// Members are shared out over host threads (member k to thread k mod T), so
// that one member's host work (a drainage recomputation, the daily global
// landsliding, lateral3's convergence loop) holds up only the members of its
// own thread while the device runs the others' chunks.
extern "C" hc_status hc_run_ensemble(hc_ctx** ctxs, int32_t m, int64_t n, int32_t flags,
                                     int64_t* done) {
  if (!ctxs || m <= 0 || n < 0) return HC_ERR_ARG;
  for (int k = 0; k < m; k++) {
    if (!ctxs[k]) return HC_ERR_ARG;
    if (done) done[k] = 0;
  }
  // longer chunks: fewer host turns per member while the others run
  for (int k = 0; k < m; k++) ctxs[k]->chunk_pref = 128;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int T = (int)std::max(1u, std::min<unsigned>((unsigned)m, std::min(hw, 32u)));
  std::vector<std::vector<int>> groups((size_t)T);
  for (int k = 0; k < m; k++) groups[(size_t)(k % T)].push_back(k);
  std::vector<hc_status> st((size_t)T, HC_OK);
  int dev = 0;
  cudaGetDevice(&dev);
  if (T == 1) return ensemble_group(ctxs, groups[0], n, flags, done);
  std::vector<std::thread> pool;
  for (int t = 0; t < T; t++)
    pool.emplace_back([&, t] {
      cudaSetDevice(dev);
      st[(size_t)t] = ensemble_group(ctxs, groups[(size_t)t], n, flags, done);
    });
  for (auto& th : pool) th.join();
  for (int t = 0; t < T; t++)
    if (st[(size_t)t] != HC_OK) return st[(size_t)t];
  return HC_OK;
}

extern "C" hc_status hc_test_bounded_waits(hc_ctx* c, int32_t spins, int32_t extra_arrivals) {
  if (!c || spins < 0 || extra_arrivals < 0) return HC_ERR_ARG;
  c->v.wait_spins = spins;
  c->v.barrier_extra = spins > 0 ? extra_arrivals : 0;
  return HC_OK;
}

extern "C" hc_status hc_get_run_stats(hc_ctx* c, int64_t* counts, double* host_ms, int32_t n) {
  if (!c || n < 0) return HC_ERR_ARG;
  if (n > HC_STAT_WET_CELL_STEPS) {
    HC_TRY(pull(c));
    c->stat_n[HC_STAT_WET_CELL_STEPS] = (int64_t)c->hdev->wet_steps;
  }
  for (int k = 0; k < n && k < HC_STAT_COUNT; k++) {
    if (counts) counts[k] = c->stat_n[k];
    if (host_ms) host_ms[k] = c->stat_ms[k];
  }
  return HC_OK;
}

// ------------------------------------------------------------------ measurement
__global__ void k_count_mask(const hc_view c, unsigned long long* n) {
  unsigned long long local = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < c.N2;
       i += (size_t)gridDim.x * blockDim.x)
    local += c.mask[i];
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(n, local);
}

extern "C" hc_status hc_bench_kernel(hc_ctx* c, const char* kernel, int32_t reps, double* avg_ms,
                                     int64_t* wet) {
  if (!c || !kernel || reps <= 0 || !avg_ms) return HC_ERR_ARG;
  const std::string k(kernel);
  unsigned long long* cnt = (unsigned long long*)((char*)c->v.red + 112);
  HC_CU(cudaMemsetAsync(cnt, 0, 8, c->s), "bench");
  k_count_mask<<<1024, 256, 0, c->s>>>(c->v, cnt);
  unsigned long long h = 0;
  HC_CU(cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, c->s), "bench");
  launch_flow_dt(c);
  cudaEvent_t e0, e1;
  HC_CU(cudaEventCreate(&e0), "bench");
  HC_CU(cudaEventCreate(&e1), "bench");
  HC_CU(cudaEventRecord(e0, c->s), "bench");
  for (int r = 0; r < reps; r++) {
    if (k == "flow_route") launch_flow_route(c, 0);
    else if (k == "depth_update") launch_depth_update(c, 0);
    else if (k == "scan_area") launch_scan_area(c, 0);
    else if (k == "entrain" && !c->v.p.hydro_only) {
      // one entrainment pass (retry flag forced on)
      launch_erode_begin(c, 0, 1.0);
      launch_erode_pass(c, 1);
    } else {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return hc_fail(c, HC_ERR_ARG, "unknown kernel %s", kernel);
    }
  }
  HC_CU(cudaEventRecord(e1, c->s), "bench");
  HC_CU(cudaEventSynchronize(e1), "bench");
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *avg_ms = ms / reps;
  if (wet) *wet = (int64_t)h;
  return HC_OK;
}

extern "C" hc_status hc_get_counters(hc_ctx* c, int64_t* launches, int64_t* h2d_bytes,
                                     int64_t* d2h_bytes) {
  if (!c) return HC_ERR_ARG;
  if (launches) *launches = c->launches;
  if (h2d_bytes) *h2d_bytes = c->h2d_bytes;
  if (d2h_bytes) *d2h_bytes = c->d2h_bytes;
  return HC_OK;
}

// One iteration of hc_run's sequence, launched phase by phase (no graph) with
// a CUDA event after each phase; ms[k] receives the time of phase k:
// 0 control+inputs, 1 flow_route, 2 depth_update, 3 scan_area,
// 4 entrainment passes, 5 apply + lateral passes + edge output,
// 6 lateral3 (when due), 7 water_flux_out, 8 slide_3.
extern "C" hc_status hc_profile_iteration(hc_ctx* c, int32_t flags, double* ms) {
  if (!c || !ms) return HC_ERR_ARG;
  if (!c->prepared) return hc_fail(c, HC_ERR_STATE, "hc_prepare must come before profiling");
  HC_TRY(pull(c));
  hc_dev* hd = c->hdev;
  hd->pause = 0;
  hd->budget = 1;
  hd->flags = flags;
  HC_TRY(push(c));
  // ev[10]: the start of the lateral3 phase, after the host has read the
  // control block (the read is not device work of any phase)
  cudaEvent_t ev[11];
  for (int k = 0; k < 11; k++) HC_CU(cudaEventCreate(&ev[k]), "profile");
  cudaEventRecord(ev[0], c->s);
  launch_control(c);
  launch_inputs(c);
  cudaEventRecord(ev[1], c->s);
  launch_flow_route(c, 1);
  cudaEventRecord(ev[2], c->s);
  launch_depth_update(c, 1);
  cudaEventRecord(ev[3], c->s);
  launch_scan_area(c, 1);
  cudaEventRecord(ev[4], c->s);
  const bool sed = !c->v.p.hydro_only;
  // the entrainment passes' device time only: the host reads the retry test
  // between passes (pass_ms sums the passes' own event pairs)
  double pass_ms = 0;
  if (sed) {
    HC_TRY(pull(c));
    cudaEvent_t p0, p1;
    HC_CU(cudaEventCreate(&p0), "profile");
    HC_CU(cudaEventCreate(&p1), "profile");
    for (int guard = 0; hd->erode_retry && hd->it_active && guard < 100000; guard++) {
      cudaEventRecord(p0, c->s);
      launch_erode_pass(c, 0);
      cudaEventRecord(p1, c->s);
      const hc_status st = pull(c);
      if (st != HC_OK) {
        cudaEventDestroy(p0);
        cudaEventDestroy(p1);
        return st;
      }
      float t = 0;
      cudaEventElapsedTime(&t, p0, p1);
      pass_ms += t;
    }
    cudaEventDestroy(p0);
    cudaEventDestroy(p1);
  }
  cudaEventRecord(ev[5], c->s);
  if (sed) {
    launch_erode_finish(c, 1);
    if (flags & HC_RUN_LATERAL) launch_lateral_check(c);
  }
  cudaEventRecord(ev[6], c->s);
  HC_TRY(pull(c));
  cudaEventRecord(ev[10], c->s);
  if (hd->pause & HC_PAUSE_LATERAL) {
    HC_TRY(run_lateral(c));
    HC_TRY(pull(c));
    hd->s.lateralcounter = hd->s.counter + (50 * hd->s.erode_mult);
    hd->pause &= ~HC_PAUSE_LATERAL;
    hd->rest_active = 1;
    HC_TRY(push(c));
  }
  cudaEventRecord(ev[7], c->s);
  launch_flux_out(c, 1, 0);
  cudaEventRecord(ev[8], c->s);
  if (sed) launch_slide3(c, 1);
  cudaEventRecord(ev[9], c->s);
  HC_CU(cudaEventSynchronize(ev[9]), "profile");
  for (int k = 0; k < 9; k++) {
    float t = 0;
    cudaEventElapsedTime(&t, k == 6 ? ev[10] : ev[k], ev[k + 1]);
    ms[k] = (k == 4) ? pass_ms : t;
  }
  for (int k = 0; k < 11; k++) cudaEventDestroy(ev[k]);
  HC_TRY(pull(c));
  HC_TRY(host_steps(c, flags));
  hd->pause &= HC_PAUSE_FINISHED;
  return push(c);
}
