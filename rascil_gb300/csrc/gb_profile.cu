// Process-wide kernel profiling: every launch of the library's kernels (and
// its cuFFT executions) can record a CUDA-event pair on the launching stream
// plus the algorithmic bytes the launch must move.  gb_profile_get()
// synchronises the events and returns per-kernel totals, so a benchmark can
// report achieved bytes / measured device time for each kernel.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gb_plan.cuh"
#include "gb_profile.cuh"

namespace gb {

namespace {
struct Pending {
  int id;
  cudaEvent_t a, b;
  double bytes, updates;
};
struct Stat {
  double ms = 0.0, bytes = 0.0, updates = 0.0;
  int64_t launches = 0;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
Stat g_stats[kProfCount];

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void drain_locked() {
  for (auto &p : g_pending) {
    cudaEventSynchronize(p.b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    g_stats[p.id].ms += ms;
    g_stats[p.id].bytes += p.bytes;
    g_stats[p.id].updates += p.updates;
    g_stats[p.id].launches += 1;
    g_pool.push_back(p.a);
    g_pool.push_back(p.b);
  }
  g_pending.clear();
}
}  // namespace

const char *kProfNames[kProfCount] = {
    "k_wrange", "k_count", "scan", "k_scatter", "k_chunks", "k_corr_image",
    "k_prep_vis", "k_grid", "cufft_inverse", "k_screen_acc", "k_finalize",
    "k_prep_image", "k_screen_pad", "cufft_forward", "k_degrid", "k_dft_components",
    "k_dft_pixels", "k_col_a_inv", "k_col_b_inv", "k_col_a_pred", "k_col_b_pred",
    "zero_margins", "k_rows_inverse", "k_rows_forward", "grid_zero",
    "k_wgrid", "k_wsums", "k_wapply", "k_wrecip", "k_rotate"};

bool prof_on() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_on;
}

ProfScope::ProfScope(int id, cudaStream_t s, double bytes, double updates)
    : id_(id), s_(s), bytes_(bytes), updates_(updates) {
  std::lock_guard<std::mutex> lk(g_mu);
  active_ = g_on;
  if (!active_) return;
  a_ = take_event();
  cudaEventRecord(a_, s_);
}

ProfScope::~ProfScope() {
  if (!active_) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t b = take_event();
  cudaEventRecord(b, s_);
  g_pending.push_back({id_, a_, b, bytes_, updates_});
  if (g_pending.size() > 4096) drain_locked();
}

}  // namespace gb

using namespace gb;

extern "C" {

int gb_profile_enable(int32_t on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_on = on != 0;
  return GB_OK;
}

int gb_profile_reset(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  drain_locked();
  for (auto &s : g_stats) s = Stat();
  return GB_OK;
}

int gb_profile_count(void) { return kProfCount; }

int gb_profile_get(int32_t i, char *name, int32_t name_len, double *total_ms,
                   int64_t *launches, double *bytes) {
  if (i < 0 || i >= kProfCount) {
    set_error("gb_profile_get: index %d out of range", i);
    return GB_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  drain_locked();
  if (name && name_len > 0) {
    strncpy(name, kProfNames[i], (size_t)name_len - 1);
    name[name_len - 1] = '\0';
  }
  if (total_ms) *total_ms = g_stats[i].ms;
  if (launches) *launches = g_stats[i].launches;
  if (bytes) *bytes = g_stats[i].bytes;
  return GB_OK;
}

int gb_profile_updates(int32_t i, double *updates) {
  if (i < 0 || i >= kProfCount || !updates) {
    set_error("gb_profile_updates: index %d out of range or NULL output", i);
    return GB_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  drain_locked();
  *updates = g_stats[i].updates;
  return GB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------
// Shared-memory peaks of this GPU, measured: the denominators of the
// gridder's (atomics) and degridder's (loads) update-rate rooflines.

namespace gb {
namespace {
constexpr int kProbeUnroll = 16;

// Conflict-free 32-bit integer atomic adds: lane l of every warp adds to
// word (warp * 32 + l) of one of four strips, 32 consecutive words per
// warp instruction (32 distinct banks).
__global__ void __launch_bounds__(kThreads) k_probe_atoms(int iters, int *out) {
  __shared__ int buf[4 * kThreads];
  for (int i = threadIdx.x; i < 4 * kThreads; i += kThreads) buf[i] = 0;
  __syncthreads();
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < kProbeUnroll; ++u)
      atomicAdd(&buf[(u & 3) * kThreads + threadIdx.x], it + u);
  }
  __syncthreads();
  if (out && threadIdx.x == 0 && buf[threadIdx.x] == 0x7fffffff) out[blockIdx.x] = buf[1];
}

// Conflict-free 8-byte loads: lane l of a warp reads float2 (base + l),
// 256 consecutive bytes per warp instruction; the sums keep the loads live.
__global__ void __launch_bounds__(kThreads) k_probe_loads(int iters, float *out) {
  __shared__ float2 buf[8 * kThreads];
  for (int i = threadIdx.x; i < 8 * kThreads; i += kThreads)
    buf[i] = make_float2((float)i, (float)(i ^ 5));
  __syncthreads();
  float ax = 0.0f, ay = 0.0f;
  for (int it = 0; it < iters; ++it) {
    const int base = (it & 7) * kThreads;
#pragma unroll
    for (int u = 0; u < kProbeUnroll; ++u) {
      const float2 v = buf[base + ((threadIdx.x + 32 * u) & (kThreads - 1))];
      ax += v.x;
      ay += v.y;
    }
  }
  if (out && ax == -1.0f && ay == -1.0f) out[blockIdx.x] = ax;
}
}  // namespace
}  // namespace gb

extern "C" {

int gb_probe_smem_peaks(double *atomics_per_s, double *loads8_per_s, void *stream) {
  if (!atomics_per_s || !loads8_per_s) {
    set_error("gb_probe_smem_peaks: NULL output");
    return GB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0, per_sm_a = 0, per_sm_l = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_a, k_probe_atoms, kThreads, 0));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_l, k_probe_loads, kThreads, 0));
  const int iters = 4096;
  const int blocks_a = sms * std::max(per_sm_a, 1), blocks_l = sms * std::max(per_sm_l, 1);
  cudaEvent_t e[3];
  for (auto &x : e) GB_CUDA(cudaEventCreate(&x));
  // warm-up, then one timed launch of each
  k_probe_atoms<<<blocks_a, kThreads, 0, s>>>(64, nullptr);
  k_probe_loads<<<blocks_l, kThreads, 0, s>>>(64, nullptr);
  GB_CUDA(cudaEventRecord(e[0], s));
  k_probe_atoms<<<blocks_a, kThreads, 0, s>>>(iters, nullptr);
  GB_CUDA(cudaEventRecord(e[1], s));
  k_probe_loads<<<blocks_l, kThreads, 0, s>>>(iters, nullptr);
  GB_CUDA(cudaEventRecord(e[2], s));
  GB_LAUNCH_CHECK("k_probe");
  GB_CUDA(cudaEventSynchronize(e[2]));
  float ta = 0.0f, tl = 0.0f;
  GB_CUDA(cudaEventElapsedTime(&ta, e[0], e[1]));
  GB_CUDA(cudaEventElapsedTime(&tl, e[1], e[2]));
  for (auto &x : e) cudaEventDestroy(x);
  const double per = (double)iters * kProbeUnroll * kThreads;
  *atomics_per_s = ta > 0.0f ? per * blocks_a / (ta * 1e-3) : 0.0;
  *loads8_per_s = tl > 0.0f ? per * blocks_l / (tl * 1e-3) : 0.0;
  return GB_OK;
}

}  // extern "C"
