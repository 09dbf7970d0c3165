// Autotuner of the launch shapes (no counterpart in the reference).
//
// k_flow_route is bound by the FP64 pipe and by the latency of its gathers;
// which register budget (blocks per multiprocessor) and grid (one resident
// wave, four waves, or the wet-list default) hides that latency best
// depends on the wet-list length and on the features of the run (erosion
// terms, Manning's n field).  hc_run times every shape of kFlowShapes on the
// live state the first time a context reaches a shape class (those
// features, and the wet-list length to a power of two), keeps the fastest,
// and caches the choice per shape class for every context of the process
// (ensemble members of like sizes tune once).  The timing launches change
// only the discharges, suspended-load fluxes and velocity directions, which
// are saved before and restored after (the kernel writes no scalar of the
// control block): the run's results do not depend on tuning.

#include "hc_internal.cuh"

#include <map>
#include <mutex>
#include <vector>

#define HC_TRY(expr)              \
  do {                            \
    hc_status st_ = (expr);       \
    if (st_ != HC_OK) return st_; \
  } while (0)

namespace {

std::mutex g_mu;
std::map<int64_t, int> g_cache;  // shape class -> shape

int64_t shape_class(const hc_ctx* c, int wet) {
  int lw = 0;
  while (lw < 40 && (1LL << (lw + 1)) <= (long long)wet) lw++;
  const hc_params& p = c->v.p;
  return ((int64_t)lw << 8) | (p.hydro_only ? 1 : 0) | (p.spatially_var_mannings ? 2 : 0) |
         (p.isSuspended[1] ? 4 : 0);
}

// the fields a k_flow_route launch writes
struct Saved {
  std::vector<std::pair<double*, size_t>> fields;  // device field, doubles
  double* copy = nullptr;
  size_t total = 0;
};

}  // namespace

hc_status autotune(hc_ctx* c, bool force) {
  if (c->flow_pinned && !force) return HC_OK;
  const int wet = c->hdev->wet_count;
  if (!force && wet < (1 << 16)) return HC_OK;  // too little work to time; the default shape
  const int64_t key = shape_class(c, wet);
  if (!force && key == c->tuned_key) return HC_OK;
  if (!force) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      if (it->second != c->flow_shape) c->graph_iters = 0;  // the graph holds the shape
      c->flow_shape = it->second;
      c->tuned_key = key;
      return HC_OK;
    }
  }
  hc_view& v = c->v;
  const size_t N2 = v.N2;
  Saved sv;
  sv.fields = {{v.qx, N2}, {v.qy, N2}};
  if (!v.p.hydro_only) {
    sv.fields.push_back({v.qxs, N2});
    sv.fields.push_back({v.qys, N2});
    sv.fields.push_back({v.vd, 4 * N2});
  }
  for (auto& f : sv.fields) sv.total += f.second;
  if (cudaMalloc(&sv.copy, sv.total * 8) != cudaSuccess) {
    cudaGetLastError();
    return HC_OK;  // no room to tune: keep the shape
  }
  cudaStream_t s = c->s;
  auto copy_fields = [&](bool save) {
    size_t off = 0;
    for (auto& f : sv.fields) {
      if (save)
        cudaMemcpyAsync(sv.copy + off, f.first, f.second * 8, cudaMemcpyDeviceToDevice, s);
      else
        cudaMemcpyAsync(f.first, sv.copy + off, f.second * 8, cudaMemcpyDeviceToDevice, s);
      off += f.second;
    }
  };
  copy_fields(true);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const cudaStream_t cs0 = c->cs;
  c->cs = s;
  // Each timed launch starts from the saved state with the L2 cache
  // flushed (a buffer larger than L2 is written first): in an iteration the
  // kernel's inputs were last touched by the previous iteration's passes,
  // so warm-cache timings (the kernel repeated) would rank the shapes by a
  // case that does not occur.
  void* flush = nullptr;
  size_t flush_bytes = 192u << 20;
  if (cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
    cudaGetLastError();
    flush = nullptr;
  }
  double best = 1e300;
  int best_k = c->flow_shape;
  for (int k = 0; k < kFlowShapeCount; k++) {
    double t = 1e300;
    launch_flow_route_shape(c, 0, k);  // the shape's first launch (module load)
    for (int round = 0; round < 3; round++) {
      copy_fields(false);
      if (flush) cudaMemsetAsync(flush, round, flush_bytes, s);
      cudaEventRecord(e0, s);
      launch_flow_route_shape(c, 0, k);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      t = std::min(t, (double)ms);
    }
    c->tune_ms[k] = t;
    if (t < best) {
      best = t;
      best_k = k;
    }
  }
  copy_fields(false);
  c->cs = cs0;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const cudaError_t e = cudaStreamSynchronize(s);
  cudaFree(sv.copy);
  if (flush) cudaFree(flush);
  if (e != cudaSuccess) return hc_cuda(c, e, "autotune");
  if (best_k != c->flow_shape) c->graph_iters = 0;
  c->flow_shape = best_k;
  c->tuned_key = key;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache[key] = best_k;
  }
  // the timing launches left the control block as it was (they are
  // ungated and write no scalar), so nothing is pushed back
  return HC_OK;
}

extern "C" hc_status hc_autotune(hc_ctx* c, int32_t force, int32_t* shape, double* ms,
                                 int32_t n) {
  if (!c || n < 0) return HC_ERR_ARG;
  if (!c->prepared) return hc_fail(c, HC_ERR_STATE, "hc_prepare must come before tuning");
  HC_TRY(ctx_pull(c));
  if (force) HC_TRY(autotune(c, true));
  if (shape) *shape = c->flow_shape;
  for (int k = 0; k < n && k < kFlowShapeCount; k++) ms[k] = c->tune_ms[k];
  return HC_OK;
}

extern "C" hc_status hc_set_launch_shape(hc_ctx* c, int32_t shape) {
  if (!c || shape < -1 || shape >= kFlowShapeCount) return HC_ERR_ARG;
  if (shape < 0) {
    c->flow_pinned = false;
    c->tuned_key = -1;  // tune again at the next hc_run
    return HC_OK;
  }
  if (shape != c->flow_shape) c->graph_iters = 0;
  c->flow_shape = shape;
  c->flow_pinned = true;
  return HC_OK;
}
