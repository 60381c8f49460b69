// Allocation-free w-range reduction.
//
// gb_plan_create finds the visibilities' w range with k_wrange, whose
// per-block partial results live in scratch memory it obtains with
// cudaMallocAsync.  Some callers cannot allocate device memory at the point
// where they need this: a host framework that hands out all device memory
// itself, or a real-time pipeline that forbids allocation after start-up.
// gb_wrange_noalloc does the same reduction with its scratch in a
// file-scope device array of fixed size instead, so it allocates nothing.
//
// Scratch: kNoAllocMaxParts partial results (min w, max w, non-finite row
// count) of kNoAllocRowsPerPart rows each -- 16384 x 3 doubles = 384 KiB,
// held by every GPU that loads this library until the process exits.  This
// bounds one call to 16384 x 4096 = 67,108,864 rows; larger inputs are
// rejected with GB_ERR_INVALID_ARG.
//
// Every call overwrites the partials it reads, so nothing needs clearing
// between calls, but all calls share the one array: calls that overlap on
// the GPU (on different streams, or from different host threads) race.
#include <mutex>

#include "gb_plan.cuh"

namespace gb {

constexpr int kNoAllocRowsPerPart = 4096;
constexpr int kNoAllocMaxParts = 16384;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_wrange_scratch[3 * kNoAllocMaxParts];

// One block per run of kNoAllocRowsPerPart rows: min/max of |w| over the
// finite rows (a w-stacking plan mirrors rows with w < 0 to -uvw, so its w
// range spans |w|) and the number of rows holding a non-finite coordinate.
__global__ void k_wrange_parts(const double *__restrict__ uvw, int64_t nrows,
                               double *__restrict__ parts) {
  const int64_t r0 = (int64_t)blockIdx.x * kNoAllocRowsPerPart;
  const int64_t r1 = min(nrows, r0 + (int64_t)kNoAllocRowsPerPart);
  double lo = INFINITY, hi = -INFINITY, bad = 0.0;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const double u = uvw[3 * r], v = uvw[3 * r + 1], w = uvw[3 * r + 2];
    if (!isfinite(u) || !isfinite(v) || !isfinite(w)) {
      bad += 1.0;
      continue;
    }
    lo = fmin(lo, fabs(w));
    hi = fmax(hi, fabs(w));
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
  }
  __shared__ double s_lo[kWarps], s_hi[kWarps], s_bad[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_lo[warp] = lo;
    s_hi[warp] = hi;
    s_bad[warp] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kWarps; ++i) {
      lo = fmin(lo, s_lo[i]);
      hi = fmax(hi, s_hi[i]);
      bad += s_bad[i];
    }
    parts[3 * blockIdx.x] = lo;
    parts[3 * blockIdx.x + 1] = hi;
    parts[3 * blockIdx.x + 2] = bad;
  }
}

// One block: combine the partials, then scale by every channel's f/c the
// way gb_plan_create does on the host, so the result is bit-identical.
__global__ void k_wrange_finish(const double *__restrict__ parts, int nparts,
                                const double *__restrict__ freq, int nchan,
                                double *__restrict__ out) {
  double lo = INFINITY, hi = -INFINITY, bad = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    lo = fmin(lo, parts[3 * i]);
    hi = fmax(hi, parts[3 * i + 1]);
    bad += parts[3 * i + 2];
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
  }
  __shared__ double s_lo[kWarps], s_hi[kWarps], s_bad[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_lo[warp] = lo;
    s_hi[warp] = hi;
    s_bad[warp] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kWarps; ++i) {
      lo = fmin(lo, s_lo[i]);
      hi = fmax(hi, s_hi[i]);
      bad += s_bad[i];
    }
    double w_lo = INFINITY, w_hi = -INFINITY, badf = 0.0;
    for (int c = 0; c < nchan; ++c) {
      const double f = freq[c];
      if (!(f > 0.0) || !isfinite(f)) {
        badf += 1.0;
        continue;
      }
      const double sc = __ddiv_rn(f, kSpeedOfLight);
      const double a = __dmul_rn(lo, sc), b = __dmul_rn(hi, sc);
      w_lo = fmin(w_lo, fmin(a, b));
      w_hi = fmax(w_hi, fmax(a, b));
    }
    out[0] = w_lo;
    out[1] = w_hi;
    out[2] = bad;
    out[3] = badf;
  }
}

// Device address of the scratch array for the current device.  Outside a
// stream capture the address is looked up on every call (with that device
// current; the lookup allocates nothing), so a context torn down and
// recreated -- cudaDeviceReset reloads the module at a new address -- is
// picked up.  Inside a capture, where the lookup is not allowed, the
// address cached by the last call outside a capture on this device is
// used; there must have been one.
static int scratch_address(cudaStream_t s, double **ptr) {
  static std::mutex mu;
  static double *cached[kNoAllocMaxDevices] = {};
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error("gb_wrange_noalloc: device ordinal %d beyond %d", dev, kNoAllocMaxDevices);
    return GB_ERR_INVALID_ARG;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  GB_CUDA(cudaStreamIsCapturing(s, &cap));
  std::lock_guard<std::mutex> lk(mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void *p = nullptr;
    GB_CUDA(cudaGetSymbolAddress(&p, g_wrange_scratch));
    cached[dev] = static_cast<double *>(p);
  } else if (!cached[dev]) {
    set_error("gb_wrange_noalloc: the first call on device %d is inside a stream capture; "
              "make one call outside a capture first", dev);
    return GB_ERR_INVALID_ARG;
  }
  *ptr = cached[dev];
  return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

int gb_wrange_noalloc(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                      int32_t nchan, double *out_dev, void *stream) {
  if (!uvw_dev || !freq_dev || !out_dev) {
    set_error("gb_wrange_noalloc: NULL argument");
    return GB_ERR_INVALID_ARG;
  }
  if (nrows <= 0 || nchan <= 0) {
    set_error("gb_wrange_noalloc: nrows and nchan must be positive (got %lld, %d)",
              (long long)nrows, nchan);
    return GB_ERR_INVALID_ARG;
  }
  const int64_t max_rows = (int64_t)kNoAllocRowsPerPart * kNoAllocMaxParts;
  if (nrows > max_rows) {
    set_error("gb_wrange_noalloc: %lld rows exceed the %lld rows its fixed scratch holds "
              "(split the call, or use gb_plan_create)",
              (long long)nrows, (long long)max_rows);
    return GB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double *parts = nullptr;
  int rc = scratch_address(s, &parts);
  if (rc) return rc;
  const int nparts = (int)((nrows + kNoAllocRowsPerPart - 1) / kNoAllocRowsPerPart);
  k_wrange_parts<<<nparts, kThreads, 0, s>>>(uvw_dev, nrows, parts);
  GB_LAUNCH_CHECK("k_wrange_parts");
  k_wrange_finish<<<1, kThreads, 0, s>>>(parts, nparts, freq_dev, nchan, out_dev);
  GB_LAUNCH_CHECK("k_wrange_finish");
  return GB_OK;
}

}  // extern "C"
