// Process-wide kernel profiling: every launch of the library's kernels (and
// its cuFFT executions) can record a CUDA-event pair on the launching stream
// plus the algorithmic bytes the launch must move.  gb_profile_get()
// synchronises the events and returns per-kernel totals, so a benchmark can
// report achieved bytes / measured device time for each kernel.
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
  double bytes;
};
struct Stat {
  double ms = 0.0, bytes = 0.0;
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

ProfScope::ProfScope(int id, cudaStream_t s, double bytes) : id_(id), s_(s), bytes_(bytes) {
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
  g_pending.push_back({id_, a_, b, bytes_});
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

}  // extern "C"
