// Plan object and launch helpers shared by gb_plan.cu, gb_invert.cu,
// gb_predict.cu and gb_capi.cu.
#pragma once

#include <cufft.h>

#include <algorithm>
#include <type_traits>
#include <string>
#include <vector>

#include "gb_internal.cuh"
#include "gb_profile.cuh"

struct gb_plan {
  gb::Geom g;
  gb_plan_params params;
  int precision;              // gb_precision
  const double *uvw = nullptr;   // caller's device arrays (used by bind)
  const double *freq = nullptr;
  gb::Quad quad;  // ES-kernel quadrature for the correction factors
  // workspace layout (byte offsets)
  size_t ws_bytes = 0;
  char *ws = nullptr;
  size_t off_items = 0, off_chunk_off = 0, off_chunks = 0, off_corr = 0,
         off_tables = 0, off_counters = 0, off_fftwork = 0, off_temp = 0;
  // bind-time temporaries (inside the temp region)
  size_t t_keys = 0, t_ranks = 0, t_counts = 0, t_offsets = 0, t_ccounts = 0,
         t_scan = 0, t_fscale = 0;
  // call-time temporaries (inside the temp region)
  size_t c_grid = 0, c_img = 0, c_cvis = 0;
  size_t max_chunks = 0;
  int nbatches = 0;
  int rem_planes = 0;
  // batched 2-D cuFFT plans: full batches of B planes, and the remainder
  cufftHandle fft_full = 0, fft_rem = 0;
  bool fft_full_ok = false, fft_rem_ok = false;
  size_t fft_work_bytes = 0;
  // column mode (FP32): the plans above are 1-D row transforms and the
  // column transforms are the library's own kernels (gb_fft.cu)
  bool col_fft = false;
  // column mode with rows of 4096 / 8192 / 16384 cells: the row transforms
  // are k_rows too (no cuFFT plan), with a (plane, row tile) occupancy mask
  bool row_fft = false;
  size_t off_rowmask = 0, off_twx = 0;
  int row_blocks = 0;
  size_t off_tprime = 0;  // [ny][nx] float64: n - 1 - tc per pixel (w-stacking)
  size_t off_coords = 0;  // shifted plans: [R][3] uvw then [C] f/c, float64
  // column mode: [ny][nx] w-screen phases as 64-bit fixed-point turns
  // (A, D), plane k's phase = A + k D mod 1; [ngy] exp(+2 pi i m / ngy)
  size_t off_screen = 0, off_twn = 0;
  bool bound = false;
  bool owns_ws = false;
  cudaStream_t last_stream = nullptr;
  int num_sms = 0;
  int grid_blocks = 0, degrid_blocks = 0;  // persistent grid sizes
  std::vector<uint32_t> slab_items;        // host copy: first item of each slab (+ total)
  std::vector<uint8_t> mask_host;          // host copy of the occupancy mask (profiling)
  // profiling only: per w-plane, grid cells in the (plane, uv tile) pairs
  // some item reaches (tile cells plus the support halo spilling into
  // tiles nothing reaches), and items whose first plane is that plane
  std::vector<int64_t> plane_cells, plane_k0;

  // Grid cells the items of planes [b0, b0 + nb) reach (0 when unknown).
  double touched_cells(int b0, int nb) const {
    if (plane_cells.empty()) return 0.0;
    double c = 0.0;
    for (int k = b0; k < b0 + nb && k < (int)plane_cells.size(); ++k) c += (double)plane_cells[k];
    return c;
  }

  // (item, plane) pairs with the item's support reaching the plane, over
  // planes [b0, b0 + nb): each is W^2 cell updates per polarisation.
  double item_planes(int b0, int nb) const {
    if (plane_k0.empty()) return 0.0;
    const int wd = g.do_w ? g.W : 1;
    double n = 0.0;
    for (int k = b0; k < b0 + nb && k < (int)plane_k0.size(); ++k)
      for (int k0 = std::max(0, k - wd + 1); k0 <= k; ++k0) n += (double)plane_k0[k0];
    return n;
  }

  // Fraction of the rows of planes [b0, b0 + nb) that visibilities reach
  // (occupancy mask; 1 without one).  Profiling byte counts only.
  double used_rows(int b0, int nb) const {
    if (mask_host.empty() || nb <= 0) return 1.0;
    int64_t used = 0;
    for (int k = b0; k < b0 + nb; ++k)
      for (int t = 0; t < g.ntv; ++t) used += mask_host[(size_t)k * g.ntv + t];
    return (double)used / ((double)nb * g.ntv);
  }

  // items whose w-slab reaches planes [b0, b0 + nb)
  uint32_t batch_items(int b0, int nb) const {
    const int lo = b0 - (g.S + g.W - 2);
    const int s_lo = lo <= 0 ? 0 : (lo + g.S - 1) / g.S;
    const int s_hi = std::min(g.nslabs - 1, (b0 + nb - 1) / g.S);
    if (slab_items.empty() || s_lo > s_hi) return 0;
    return slab_items[s_hi + 1] - slab_items[s_lo];
  }

  // Device status word (kernels OR error bits in; gb_plan_device_status reads it).
  uint32_t *status_word() const { return at<uint32_t>(off_counters) + 2 * nbatches; }

  template <typename T> T *at(size_t off) const {
    return reinterpret_cast<T *>(ws + off);
  }
};

namespace gb {

// Host planning (no device work).  Returns GB_OK or GB_ERR_INVALID_ARG.
int plan_geometry(const gb_plan_params *p, double w_lo, double w_hi, Geom &g);

// Sizes of one complex / real element for the plan's precision.
inline size_t cplx_bytes(int precision) { return precision == GB_FP64 ? 16 : 8; }
inline size_t real_bytes(int precision) { return precision == GB_FP64 ? 8 : 4; }

// Exclusive scan of n uint32 counts into out[0..n] (out[n] = total).
int scan_exclusive(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp,
                   cudaStream_t s);
size_t scan_tmp_words(int64_t n);

// Invert / predict drivers (gb_invert.cu / gb_predict.cu).
int run_ms2dirty(gb_plan *p, const void *vis, int npv, const void *wgt,
                 const void *flags, int flags_type, const PolMat &pm, int psf,
                 void *dirty, int layout, double *sumwt, cudaStream_t s);
int run_dirty2ms(gb_plan *p, const void *dirty, int layout, const void *wgt,
                 const PolMat &pm, int npv, void *vis, cudaStream_t s);
int setup_tile_kernels(gb_plan *p);

// The same drivers in steps, for a batch of plans that interleaves them
// (gb_batch.cu).  Invert: begin, then per w-plane batch bi zero -> grid ->
// transform, then end.  Predict: begin, then per batch transform -> degrid.
int inv_begin(gb_plan *p, const void *vis, int npv, const void *wgt, const void *flags,
              int ftype, const PolMat &pm, int psf, double *sumwt, cudaStream_t s);
int inv_zero(gb_plan *p, int bi, cudaStream_t s);
int inv_transform(gb_plan *p, int bi, cudaStream_t s);
int inv_end(gb_plan *p, void *dirty, int layout, cudaStream_t s);
int pred_begin(gb_plan *p, const void *dirty, int layout, cudaStream_t s);
int pred_transform(gb_plan *p, int bi, cudaStream_t s);

// Polarisation matrix from a host array of nout x nin complex (re, im
// interleaved; NULL = identity, which needs nout == nin).
int make_polmat(const double *host, int nout, int nin, PolMat &pm);

// One plan's batch of w-planes in a multi-plan gridding or degridding launch
// (FP32 form), passed to the kernel by value.
constexpr int kMaxJobs = 16;
struct GridJob {
  Geom g;
  const void *items;          // ItemF, bucket order
  const void *cvis;           // gridding: per-item values; degridding: unused
  const Chunk *chunks;
  const uint32_t *chunk_off;  // per-bucket chunk offsets (device)
  void *grid;                 // the batch's planes
  int b0, nb;                 // the batch's w-planes
  // degridding only
  void *vis;                  // [nrows][nchan][npv] complex64 output
  int npv, pad;
  const float *wgt;           // or null
  RowPerm rp;
};
struct GridJobs {
  int n;
  GridJob job[kMaxJobs];
};
int grid_job(gb_plan *p, int bi, GridJob &jb);
void grid_job_counts(const gb_plan *p, int bi, double *bytes, double *updates);
int launch_grid_jobs(const GridJobs &jobs, int num_sms, uint32_t *counter, double bytes,
                     double updates, cudaStream_t s);
int degrid_job(gb_plan *p, int bi, void *vis, int npv, GridJob &jb);
void degrid_job_counts(const gb_plan *p, int bi, int npv, double *bytes, double *updates);
int launch_degrid_jobs(const GridJobs &jobs, const PolMat &pm, int num_sms, uint32_t *counter,
                       double bytes, double updates, cudaStream_t s);

}  // namespace gb

#define GB_CUDA(call)                                          \
  do {                                                         \
    cudaError_t e__ = (call);                                  \
    if (e__ != cudaSuccess) return gb::cuda_fail(e__, #call);  \
  } while (0)

// Launch check.  With RASCIL_GB300_SYNC_CHECK=1 in the environment every
// launch is also synchronised, so an asynchronous fault names its kernel.
namespace gb {
bool sync_check_enabled();
}
#define GB_LAUNCH_CHECK(what)                                           \
  do {                                                                  \
    cudaError_t e__ = cudaGetLastError();                               \
    if (e__ == cudaSuccess && gb::sync_check_enabled())                 \
      e__ = cudaDeviceSynchronize();                                    \
    if (e__ != cudaSuccess) return gb::cuda_fail(e__, what);            \
  } while (0)
