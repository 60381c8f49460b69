// Planning and the device-side bucket sort.
//
// gb_plan_create  -> w range on the device (one sync), host geometry,
//                    cuFFT plans (no device memory), workspace layout.
// gb_plan_bind    -> count items per (w-slab, uv-tile) bucket with
//                    warp-aggregated atomics, exclusive scan, scatter one
//                    compact record per item into bucket order, cut the
//                    buckets into work chunks, build the correction image.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "es_table.h"
#include "gb_fft.cuh"
#include "gb_plan.cuh"

namespace gb {

static thread_local char tl_error[512] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(tl_error, sizeof(tl_error), fmt, ap);
  va_end(ap);
}

int cuda_fail(cudaError_t e, const char *what) {
  set_error("CUDA error %s (%d) in %s", cudaGetErrorString(e), (int)e, what);
  return GB_ERR_CUDA;
}

const char *last_error() { return tl_error; }

bool sync_check_enabled() {
  static const bool on = [] {
    const char *v = getenv("RASCIL_GB300_SYNC_CHECK");
    return v && v[0] == '1';
  }();
  return on;
}

// ---------------------------------------------------------------------
// Host planning

static int good_size(int n) {
  if (n < 16) n = 16;
  for (;; ++n) {
    if (n & 1) continue;
    int m = n;
    for (int f : {2, 3, 5, 7})
      while (m % f == 0) m /= f;
    if (m == 1) return n;
  }
}

static int plan_geometry_sigma(const gb_plan_params *p, double w_lo, double w_hi, double sigma,
                               Geom &g);

// Cost model of one direction (invert or predict) of a plan, in seconds on
// GB300, for choosing the grid oversampling when the caller leaves it at 0
// (ducc0 makes the same choice internally from a cost model): gridding work
// per (item, w-plane its support reaches, polarisation), growing as W^2,
// plus per-plane transform work per grid cell and polarisation -- the
// library's pruned row/column transforms where they apply, batched 2-D
// cuFFT plans with separate zeroing and screen passes otherwise.  Constants
// measured on GB300: per update on the LOW-like workload (k_grid and
// k_degrid_warp, mean of the two directions), per cell for the column-mode
// passes there; the FP32 cuFFT-path cell cost is set so that the 256
// snapshots of the batched workload (1024^2 and 2048^2 images, mostly empty
// w-planes) keep sigma 2, which measured 12 % faster over the list than
// sigma 1.5 on 3072^2 / 1536^2 cuFFT grids.
constexpr double kCostItemPlane[2] = {6.6e-11, 2.5e-9};  // FP32, FP64 (at W = 7)
constexpr double kCostCellColumns = 4.5e-12;
constexpr double kCostCellCufft[2] = {1.3e-11, 1.8e-11};

static bool columns_apply(const gb_plan_params *p, const Geom &g) {
  int n1, n2;
  return p->precision == GB_FP32 && p->fft_mode != GB_FFT_CUFFT_2D && g.ngy == 2 * g.ny &&
         (g.ngx - g.nx) % 4 == 0 && column_split(g.ngy, n1, n2);
}

static double plan_cost(const gb_plan_params *p, const Geom &g) {
  const int f = p->precision == GB_FP64 ? 1 : 0;
  const double items = (double)p->nrows * (double)p->nchan;
  const double wp = g.do_w ? g.W : 1;
  const double grid = items * g.NP * wp * (g.W * g.W / 49.0) * kCostItemPlane[f];
  const double cell = columns_apply(p, g) ? kCostCellColumns : kCostCellCufft[f];
  return grid + (double)g.nplanes * g.NP * (double)g.ngx * (double)g.ngy * cell;
}

int plan_geometry(const gb_plan_params *p, double w_lo, double w_hi, Geom &g) {
  if (!p) {
    set_error("params is NULL");
    return GB_ERR_INVALID_ARG;
  }
  if (p->sigma > 0.0) return plan_geometry_sigma(p, w_lo, w_hi, p->sigma, g);
  // sigma 0: the tabulated oversampling of least modelled cost among those
  // the form allows; 2.0 unless another is at least 10 % cheaper
  // (power-of-two grids for power-of-two images, the library's own
  // transforms)
  static const double kSigmas[] = {2.0, 1.75, 1.5, 1.25};
  double best = 0.0;
  bool found = false;
  for (double sg : kSigmas) {
    Geom t;
    if (plan_geometry_sigma(p, w_lo, w_hi, sg, t) != GB_OK) continue;
    if (p->fft_mode == GB_FFT_COLUMNS && !columns_apply(p, t)) continue;
    const double c = plan_cost(p, t) * (sg == 2.0 ? 0.9 : 1.0);
    if (!found || c < best) {
      best = c;
      g = t;
      found = true;
    }
  }
  if (!found) return plan_geometry_sigma(p, w_lo, w_hi, 2.0, g);  // for its error message
  set_error("");
  return GB_OK;
}

static int plan_geometry_sigma(const gb_plan_params *p, double w_lo, double w_hi, double sigma,
                               Geom &g) {
  if (p->nrows <= 0 || p->nchan <= 0) {
    set_error("nrows and nchan must be positive (got %lld, %d)", (long long)p->nrows,
              p->nchan);
    return GB_ERR_INVALID_ARG;
  }
  if (p->npol != 1 && p->npol != 2 && p->npol != 4) {
    set_error("npol must be 1, 2 or 4 (got %d)", p->npol);
    return GB_ERR_INVALID_ARG;
  }
  if (p->npix_x < 16 || p->npix_y < 16 || (p->npix_x & 1) || (p->npix_y & 1)) {
    set_error("npix_x and npix_y must be even and >= 16 (got %d, %d)", p->npix_x,
              p->npix_y);
    return GB_ERR_INVALID_ARG;
  }
  if (!(p->pixsize_x > 0.0) || !(p->pixsize_y > 0.0) || !std::isfinite(p->pixsize_x) ||
      !std::isfinite(p->pixsize_y)) {
    set_error("pixel sizes must be positive and finite");
    return GB_ERR_INVALID_ARG;
  }
  if (p->precision != GB_FP32 && p->precision != GB_FP64) {
    set_error("precision must be GB_FP32 or GB_FP64");
    return GB_ERR_INVALID_ARG;
  }
  if (!(p->epsilon > 0.0) || !(p->epsilon < 1.0)) {
    set_error("epsilon must be in (0, 1) (got %g)", p->epsilon);
    return GB_ERR_INVALID_ARG;
  }
  if (p->precision == GB_FP32 && p->epsilon < 1e-6) {
    set_error("epsilon %g is below what the FP32 form can reach (1e-6); use GB_FP64",
              p->epsilon);
    return GB_ERR_INVALID_ARG;
  }
  // At sigma 1.25 the kernel's Fourier transform falls to 0.7 % of its peak at
  // the image edge, so the correction multiplies edge pixels by up to ~150 per
  // dimension: FP32 grid rounding (and the run-to-run order of its float
  // atomics) then reaches 1e-4 there.  The FP32 form keeps sigma >= 1.5 below
  // epsilon 1e-4.
  if (p->precision == GB_FP32 && sigma < 1.5 && p->epsilon < 1e-4) {
    set_error("sigma %g with epsilon %g: the FP32 form needs sigma >= 1.5 (its grid rounding, "
              "amplified by the edge correction, exceeds epsilon); use GB_FP64 or sigma >= 1.5",
              sigma, p->epsilon);
    return GB_ERR_INVALID_ARG;
  }
  if (!std::isfinite(w_lo) || !std::isfinite(w_hi) || w_hi < w_lo) {
    set_error("invalid w range [%g, %g]", w_lo, w_hi);
    return GB_ERR_INVALID_ARG;
  }
  memset(&g, 0, sizeof(g));
  const int ndim = p->do_wstacking ? 3 : 2;
  int W = 0;
  double beta = 0.0;
  bool sigma_known = false;
  for (int i = 0; i < kGbEsTableSize; ++i) {
    const GbEsEntry &e = kGbEsTable[i];
    if (std::fabs(e.sigma - sigma) > 1e-9) continue;
    sigma_known = true;
    if (p->support > 0) {
      if (e.support == p->support) {
        W = e.support;
        beta = e.beta;
        break;
      }
    } else if (ndim * e.error <= p->epsilon) {
      W = e.support;
      beta = e.beta;
      break;
    }
  }
  if (!sigma_known) {
    set_error("sigma %g not tabulated (use 1.25, 1.5, 1.75 or 2.0)", sigma);
    return GB_ERR_INVALID_ARG;
  }
  if (W == 0) {
    if (p->support > 0)
      set_error("support %d not tabulated (4..16)", p->support);
    else
      set_error("epsilon %g not reachable with sigma %g", p->epsilon, sigma);
    return GB_ERR_INVALID_ARG;
  }
  g.nx = p->npix_x;
  g.ny = p->npix_y;
  g.dx = p->pixsize_x;
  g.dy = p->pixsize_y;
  g.W = W;
  g.beta = beta;
  g.sigma = sigma;
  g.do_w = p->do_wstacking ? 1 : 0;
  g.ngx = good_size(std::max((int)std::ceil(sigma * p->npix_x), 2 * W));
  g.ngy = good_size(std::max((int)std::ceil(sigma * p->npix_y), 2 * W));
  const double xm = 0.5 * p->npix_x * p->pixsize_x;
  const double ym = 0.5 * p->npix_y * p->pixsize_y;
  const double r2 = xm * xm + ym * ym;
  if (!(r2 < 1.0)) {
    set_error("field of view reaches the horizon (l^2 + m^2 = %g)", r2);
    return GB_ERR_INVALID_ARG;
  }
  if (g.do_w) {
    const double tmin = -r2 / (1.0 + std::sqrt(1.0 - r2));
    const double tmax = 0.0;
    g.tc = 0.5 * (tmin + tmax);
    const double half = 0.5 * (tmax - tmin);
    g.dw = 1.0 / (2.0 * sigma * half);
    g.w_lo = w_lo;
    g.w_hi = w_hi;
    const double span = std::ceil((w_hi - w_lo) / g.dw);
    if (span > 1e6) {
      set_error("w range needs %g w-planes (> 1e6)", span);
      return GB_ERR_INVALID_ARG;
    }
    g.nplanes = (int)span + W;
  } else {
    g.tc = 0.0;
    g.dw = 1.0;
    g.w_lo = 0.0;
    g.w_hi = 0.0;
    g.nplanes = 1;
  }
  int T = p->tile > 0 ? p->tile : (p->precision == GB_FP64 ? 16 : 32);
  if (T < 4 || T > kMaxTile) {
    set_error("tile %d outside [4, %d]", T, kMaxTile);
    return GB_ERR_INVALID_ARG;
  }
  int S = p->slab > 0 ? p->slab : 4;
  if (S > kMaxSlab) {
    set_error("slab %d outside [1, %d]", S, kMaxSlab);
    return GB_ERR_INVALID_ARG;
  }
  g.T = T;
  g.S = S;
  g.ntu = (g.ngx + T - 1) / T;
  g.ntv = (g.ngy + T - 1) / T;
  g.nslabs = (g.nplanes + S - 1) / S;
  g.nbuckets = (int64_t)g.nslabs * g.ntu * g.ntv;
  // the sort keys order items by bucket, then by first w-plane inside the
  // slab: nbuckets x S keys
  if (g.nbuckets * S >= (int64_t)0xffffffffLL) {
    set_error("too many buckets (%lld x %d w-planes per slab)", (long long)g.nbuckets, S);
    return GB_ERR_INVALID_ARG;
  }
  const int64_t nitems = p->nrows * (int64_t)p->nchan;
  if (nitems >= (int64_t)0xffffffffLL) {
    set_error("nrows * nchan = %lld exceeds 2^32 - 1; split the call", (long long)nitems);
    return GB_ERR_INVALID_ARG;
  }
  g.R = p->nrows;
  g.C = p->nchan;
  g.NP = p->npol;
  g.nitems = (uint32_t)nitems;
  for (int k = 0; k < 3; ++k) {
    if (!std::isfinite(p->phase_shift[k])) {
      set_error("phase_shift[%d] = %g is not finite", k, p->phase_shift[k]);
      return GB_ERR_INVALID_ARG;
    }
    g.shift[k] = p->phase_shift[k];
  }
  g.shifted = g.shift[0] != 0.0 || g.shift[1] != 0.0 || g.shift[2] != 0.0;
  const int64_t budget =
      p->grid_budget_bytes > 0 ? p->grid_budget_bytes : (int64_t)32 << 30;
  const int64_t per_plane =
      (int64_t)g.NP * g.ngx * g.ngy * (int64_t)cplx_bytes(p->precision);
  int64_t B = p->planes_per_batch > 0 ? (int64_t)p->planes_per_batch : budget / per_plane;
  if (B < 1) B = 1;
  if (B > g.nplanes) B = g.nplanes;
  g.B = (int)B;
  g.nquad = std::min(kMaxQuad, 2 * W + 16);
  return GB_OK;
}

// ---------------------------------------------------------------------
// Scan

constexpr int kScanItems = 8;
constexpr int kScanTile = kThreads * kScanItems;

__global__ void k_scan_tiles(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                             int64_t n_in, int64_t n_out, uint32_t *__restrict__ tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n_in) ? in[base + i] : 0u;
    s += v[i];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __shared__ uint32_t wsum[kWarps];
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = lane < kWarps ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < kWarps; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kWarps) wsum[lane] = t;
  }
  __syncthreads();
  const uint32_t warp_off = warp ? wsum[warp - 1] : 0u;
  uint32_t run = warp_off + x - s;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n_out) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == kThreads - 1) tile_sums[blockIdx.x] = warp_off + x;
}

__global__ void k_scan_add(uint32_t *__restrict__ out, int64_t n_out,
                           const uint32_t *__restrict__ offs) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  const uint32_t add = offs[blockIdx.x];
  for (int i = threadIdx.x; i < kScanTile; i += kThreads) {
    if (base + i < n_out) out[base + i] += add;
  }
}

size_t scan_tmp_words(int64_t n) {
  size_t words = 0;
  int64_t m = n + 1;
  while (true) {
    const int64_t tiles = (m + kScanTile - 1) / kScanTile;
    if (tiles <= 1) break;
    words += (size_t)tiles + (size_t)(tiles + 1) + 8;
    m = tiles + 1;  // next level scans `tiles` sums into tiles+1 outputs
  }
  return words + 64;
}

// out[0..n] = exclusive scan of in[0..n-1], out[n] = total.
int scan_exclusive(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp,
                   cudaStream_t s) {
  const int64_t n_out = n + 1;
  const int64_t tiles = (n_out + kScanTile - 1) / kScanTile;
  uint32_t *sums = tmp;
  k_scan_tiles<<<(unsigned)tiles, kThreads, 0, s>>>(in, out, n, n_out, sums);
  GB_LAUNCH_CHECK("k_scan_tiles");
  if (tiles > 1) {
    uint32_t *sums_scanned = sums + tiles;
    int rc = scan_exclusive(sums, sums_scanned, tiles, sums_scanned + tiles + 1 + 8, s);
    if (rc) return rc;
    k_scan_add<<<(unsigned)tiles, kThreads, 0, s>>>(out, n_out, sums_scanned);
    GB_LAUNCH_CHECK("k_scan_add");
  }
  return GB_OK;
}

// ---------------------------------------------------------------------
// w range

// Range of w (of |w| when rows with w < 0 are mirrored, row_flipped) over
// the finite rows, and the count of rows with a non-finite coordinate.
__global__ void k_wrange(const double *__restrict__ uvw, int64_t nrows, int mirror,
                         double *__restrict__ part) {
  double lo = INFINITY, hi = -INFINITY, bad = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const double u = uvw[3 * r], v = uvw[3 * r + 1], w = uvw[3 * r + 2];
    if (!isfinite(u) || !isfinite(v) || !isfinite(w)) {
      bad += 1.0;
      continue;
    }
    const double wm = mirror ? fabs(w) : w;
    lo = fmin(lo, wm);
    hi = fmax(hi, wm);
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
    part[3 * blockIdx.x] = lo;
    part[3 * blockIdx.x + 1] = hi;
    part[3 * blockIdx.x + 2] = bad;
  }
}

// ---------------------------------------------------------------------
// Bucket sort

// Sort key of an item: its bucket, then its first w-plane inside the slab,
// so a bucket's items run in order of first w-plane (the kernels then find
// the items reaching one w-plane as one contiguous run, and the lanes of a
// warp reach the same w-planes).
__host__ __device__ inline uint32_t sort_key(const Geom &g, const Coord &o) {
  return bucket_of(g, o) * (uint32_t)g.S + (uint32_t)(o.k0 % g.S);
}

// f/c per channel, once per plan: the per-item coordinates multiply by it
// (one IEEE division per channel, as the oracle forms freq / c, instead of
// one per (row, channel) item).
__global__ void k_freq_scale(const double *__restrict__ freq, int nchan,
                             double *__restrict__ fscale) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nchan) fscale[c] = __ddiv_rn(freq[c], kSpeedOfLight);
}

__global__ void k_count(const Geom g, const double *__restrict__ uvw,
                        const double *__restrict__ fscale, uint32_t *__restrict__ counts,
                        uint32_t *__restrict__ keys, uint32_t *__restrict__ ranks) {
  const int lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < g.nitems; base += stride) {
    const uint64_t i = base + threadIdx.x;
    const bool active = i < g.nitems;
    uint32_t key = 0xffffffffu;
    if (active) {
      Coord o;
      item_coord(g, uvw, fscale, (uint32_t)i, o);
      key = sort_key(g, o);
    }
    // warp-aggregated increment: one atomic per distinct key in the warp
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    const uint32_t below = __popc(peers & ((1u << lane) - 1u));
    uint32_t start = 0;
    if (lane == leader && active) start = atomicAdd(&counts[key], (uint32_t)__popc(peers));
    start = __shfl_sync(peers, start, leader);
    if (active) {
      keys[i] = key;
      ranks[i] = start + below;
    }
  }
}

template <typename R>
__global__ void k_scatter(const Geom g, const double *__restrict__ uvw,
                          const double *__restrict__ fscale, const uint32_t *__restrict__ keys,
                          const uint32_t *__restrict__ ranks,
                          const uint32_t *__restrict__ offsets,
                          typename Traits<R>::Item *__restrict__ items) {
  using Item = typename Traits<R>::Item;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.nitems; i += stride) {
    Coord o;
    item_coord(g, uvw, fscale, (uint32_t)i, o);
    const uint32_t pos = offsets[keys[i]] + ranks[i];
    Item it;
    it.idx = (uint32_t)i;
    const uint32_t lu = (uint32_t)(o.p0 % g.T), lv = (uint32_t)(o.q0 % g.T);
    const uint32_t lk = (uint32_t)(o.k0 % g.S);
    it.loc = lu | (lv << 8) | (lk << 16) | (o.flip ? kLocFlip : 0u);
    it.du = (R)o.du;
    it.dv = (R)o.dv;
    it.dwf = (R)o.dwf;
    if (g.do_w || g.shifted) {
      // exp(-2 pi i (w tc - (u, v, w) . shift)), reduced in FP64 before the sincos
      const double turns = item_turns(g, uvw, fscale, (uint32_t)i, g.shifted);
      R s, c;
      sincos_2pi((R)turns, &s, &c);
      it.ph.x = c;
      it.ph.y = -s;
    } else {
      it.ph.x = (R)1;
      it.ph.y = (R)0;
    }
    if constexpr (sizeof(R) == 4) it.pad = 0.0f;
    items[pos] = it;
  }
}

// offsets[] is over sort keys (S per bucket): bucket b's items are
// [offsets[b S], offsets[(b + 1) S]).
__global__ void k_chunk_counts(const uint32_t *__restrict__ offsets, int S, int64_t nbuckets,
                               uint32_t *__restrict__ ccounts) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbuckets; b += stride) {
    const uint32_t n = offsets[(b + 1) * S] - offsets[b * S];
    ccounts[b] = (n + kChunkItems - 1) / kChunkItems;
  }
}

__global__ void k_emit_chunks(const uint32_t *__restrict__ offsets, int S,
                              const uint32_t *__restrict__ chunk_off, int64_t nbuckets,
                              Chunk *__restrict__ chunks) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbuckets; b += stride) {
    const uint32_t lo = offsets[b * S], hi = offsets[(b + 1) * S];
    uint32_t c = chunk_off[b];
    for (uint32_t s = lo; s < hi; s += kChunkItems, ++c) {
      Chunk ch;
      ch.begin = s;
      ch.end = min(hi, s + (uint32_t)kChunkItems);
      ch.bucket = (uint32_t)b;
      ch.pad = 0;
      chunks[c] = ch;
    }
  }
}

__global__ void k_slab_items(const uint32_t *__restrict__ offsets, int nslabs, int64_t ntiles,
                             int S, uint32_t *__restrict__ out) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s <= nslabs; s += gridDim.x * blockDim.x)
    out[s] = offsets[(int64_t)s * ntiles * S];
}

// Correction image [ny][nx]: 1/(phihat_u phihat_v) and, with w-stacking,
// 1/(phihat_w(dw t') n).  phihat_w by Gauss-Legendre quadrature of the
// (even) kernel on [0, W/2].

template <typename R>
__global__ void k_corr_image(const Geom g, const double *__restrict__ cu,
                             const double *__restrict__ cv, const Quad quad,
                             R *__restrict__ corr, double *__restrict__ tprime,
                             ulonglong2 *__restrict__ screen) {
  const int64_t npix = (int64_t)g.nx * g.ny;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix; i += stride) {
    const int iy = (int)(i / g.nx), ix = (int)(i - (int64_t)iy * g.nx);
    double f = cu[ix] * cv[iy];
    if (g.do_w) {
      const double t = pixel_nm1(g, ix, iy);
      tprime[i] = t - g.tc;
      if (screen) {
        // plane k sits at w_k = c0 + k dw: phase_k = c0 t' + k (dw t') turns
        const double c0 = g.w_lo - 0.5 * g.W * g.dw;
        screen[i] = make_ulonglong2(fixed_turns(c0 * (t - g.tc)), fixed_turns(g.dw * (t - g.tc)));
      }
      // phihat_w(dw t') by quadrature, in the form's own precision
      const R nu = (R)(g.dw * (t - g.tc));
      R ph = (R)0;
      for (int q = 0; q < quad.n; ++q) {
        R s, c;
        sincos_2pi((R)quad.x[q] * nu, &s, &c);
        ph += (R)quad.w[q] * c;
      }
      f = f / (2.0 * (double)ph * (1.0 + t));
    }
    corr[i] = (R)f;
  }
}

// Occupancy of (w-plane, row tile): a chunk's items reach planes
// [slab S, slab S + S + W - 1) and rows [tv T, tv T + T + W - 1) (mod ngy).
__global__ void k_row_mask(const Geom g, const Chunk *__restrict__ chunks,
                           const uint32_t *__restrict__ chunk_off, uint8_t *__restrict__ mask) {
  const uint32_t nch = chunk_off[g.nbuckets];
  const int ntiles = g.ntu * g.ntv;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nch; c += gridDim.x * blockDim.x) {
    const uint32_t bucket = chunks[c].bucket;
    const int slab = (int)(bucket / (uint32_t)ntiles);
    const int tv = (int)(bucket - (uint32_t)slab * ntiles) / g.ntu;
    const int k_lo = slab * g.S, k_hi = min(k_lo + g.S + g.W - 1, g.nplanes);
    const int r_lo = tv * g.T, r_hi = tv * g.T + g.T + g.W - 2;  // inclusive
    for (int k = k_lo; k < k_hi; ++k) {
      for (int r = r_lo; r <= r_hi + g.T - 1; r += g.T) {
        int rr = min(r, r_hi);
        while (rr >= g.ngy) rr -= g.ngy;
        mask[(int64_t)k * g.ntv + rr / g.T] = 1;
      }
    }
  }
}

// Profiling statistics (one thread per chunk): mark every (w-plane, uv
// tile) pair the chunk's items reach and count items per first w-plane.
template <typename Item>
__global__ void k_plane_stats(const Geom g, const Item *__restrict__ items,
                              const Chunk *__restrict__ chunks,
                              const uint32_t *__restrict__ chunk_off, uint8_t *__restrict__ tmask,
                              unsigned long long *__restrict__ k0_count) {
  const uint32_t nch = chunk_off[g.nbuckets];
  const int ntiles = g.ntu * g.ntv;
  const int wd = g.do_w ? g.W : 1;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nch; c += gridDim.x * blockDim.x) {
    const Chunk ch = chunks[c];
    const int slab = (int)(ch.bucket / (uint32_t)ntiles);
    const int tile = (int)(ch.bucket - (uint32_t)slab * ntiles);
    int lo = 1 << 30, hi = -1;
    uint32_t cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t j = ch.begin; j < ch.end; ++j) {
      const int lk = (int)((items[j].loc >> 16) & 0xffu);
      lo = min(lo, lk);
      hi = max(hi, lk);
      if (lk < 8)
        ++cnt[lk];
      else
        atomicAdd(&k0_count[slab * g.S + lk], 1ull);
    }
    for (int lk = 0; lk < 8; ++lk)
      if (cnt[lk]) atomicAdd(&k0_count[slab * g.S + lk], (unsigned long long)cnt[lk]);
    for (int k = slab * g.S + lo; hi >= 0 && k < min(slab * g.S + hi + wd, g.nplanes); ++k)
      tmask[(int64_t)k * ntiles + tile] = 1;
  }
}

// Cells per w-plane in the marked tiles: T x T per tile (clipped at the
// grid's edge) plus the W - 1 halo strips and corner that spill into an
// unmarked neighbour (support footprints start inside their tile).
__global__ void k_plane_cells(const Geom g, const uint8_t *__restrict__ tmask,
                              unsigned long long *__restrict__ cells) {
  const int ntiles = g.ntu * g.ntv;
  for (int k = blockIdx.y; k < g.nplanes; k += gridDim.y) {
    const uint8_t *m = tmask + (int64_t)k * ntiles;
    unsigned long long acc = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles;
         t += gridDim.x * blockDim.x) {
      if (!m[t]) continue;
      const int tv = t / g.ntu, tu = t - tv * g.ntu;
      const int wu = min(g.T, g.ngx - tu * g.T), wv = min(g.T, g.ngy - tv * g.T);
      const int tu1 = tu + 1 == g.ntu ? 0 : tu + 1, tv1 = tv + 1 == g.ntv ? 0 : tv + 1;
      const int h = g.W - 1;
      acc += (unsigned long long)wu * wv;
      if (!m[tv * g.ntu + tu1]) acc += (unsigned long long)h * wv;
      if (!m[tv1 * g.ntu + tu]) acc += (unsigned long long)wu * h;
      if (!m[tv1 * g.ntu + tu1]) acc += (unsigned long long)h * h;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&cells[k], acc);
  }
}

// Host copies of the per-plane statistics (profiling only; synchronises).
template <typename Item>
static int plane_stats(gb_plan *p, cudaStream_t s) {
  const Geom &g = p->g;
  const int64_t ntiles = (int64_t)g.ntu * g.ntv;
  const size_t mbytes = (size_t)g.nplanes * (size_t)ntiles;
  p->plane_cells.clear();
  p->plane_k0.clear();
  if (mbytes > ((size_t)1 << 30)) return GB_OK;  // too large to be worth it: no statistics
  uint8_t *tmask = nullptr;
  unsigned long long *cnt = nullptr;
  GB_CUDA(cudaMallocAsync((void **)&tmask, mbytes, s));
  GB_CUDA(cudaMallocAsync((void **)&cnt, 16 * (size_t)g.nplanes, s));
  GB_CUDA(cudaMemsetAsync(tmask, 0, mbytes, s));
  GB_CUDA(cudaMemsetAsync(cnt, 0, 16 * (size_t)g.nplanes, s));
  const unsigned cb = (unsigned)std::min<int64_t>(
      ((int64_t)p->max_chunks + kThreads - 1) / kThreads, (int64_t)p->num_sms * 16);
  k_plane_stats<Item><<<cb, kThreads, 0, s>>>(g, p->at<Item>(p->off_items),
                                              p->at<Chunk>(p->off_chunks),
                                              p->at<uint32_t>(p->off_chunk_off), tmask,
                                              cnt + g.nplanes);
  GB_LAUNCH_CHECK("k_plane_stats");
  const dim3 grid((unsigned)std::min<int64_t>((ntiles + kThreads - 1) / kThreads, 64),
                  (unsigned)std::min(g.nplanes, 65535));
  k_plane_cells<<<grid, kThreads, 0, s>>>(g, tmask, cnt);
  GB_LAUNCH_CHECK("k_plane_cells");
  std::vector<unsigned long long> h(2 * (size_t)g.nplanes);
  GB_CUDA(cudaMemcpyAsync(h.data(), cnt, 16 * (size_t)g.nplanes, cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(tmask, s);
  cudaFreeAsync(cnt, s);
  GB_CUDA(cudaStreamSynchronize(s));
  p->plane_cells.assign(h.begin(), h.begin() + g.nplanes);
  p->plane_k0.assign(h.begin() + g.nplanes, h.end());
  return GB_OK;
}

// exp(+2 pi i m / n), m < n, rounded from FP64.
__global__ void k_twiddles(int n, float2 *__restrict__ tw) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < n) {
    double sn, cs;
    sincospi(2.0 * (double)m / (double)n, &sn, &cs);
    tw[m] = make_float2((float)cs, (float)sn);
  }
}

// Host: Gauss-Legendre nodes on [-1, 1] (Newton on the Legendre recurrence).
static void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = 0.0;
      for (int j = 1; j <= n; ++j) {
        const double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p2) / j;
      }
      dp = n * (z * p0 - p1) / (z * z - 1.0);
      const double dz = p0 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

static double es_host(double x, double beta) {
  const double t = 1.0 - x * x;
  return t > 0.0 ? std::exp(beta * (std::sqrt(t) - 1.0)) : 0.0;
}

// Half-interval quadrature of the ES kernel (nodes in cells, weights times
// kernel values).
static void make_quadrature(const Geom &g, Quad &q) {
  const int nq = g.nquad;
  std::vector<double> x2, w2;
  gauss_legendre(2 * nq, x2, w2);
  q.n = nq;
  for (int i = 0; i < nq; ++i) {
    const double xn = x2[nq + i];  // positive half
    q.x[i] = xn * 0.5 * g.W;
    q.w[i] = w2[nq + i] * 0.5 * g.W * es_host(xn, g.beta);
  }
}

// cu[ix] = 1/phihat((ix - nx/2)/ngx) and cv[iy] likewise, FP64 on the device
// (keeps the plan's bind free of host copies, so it can be graph-captured).
__global__ void k_corr_1d(const Geom g, const Quad quad, double *__restrict__ cu,
                          double *__restrict__ cv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.nx + g.ny;
       i += gridDim.x * blockDim.x) {
    const double nu = i < g.nx ? (double)(i - g.nx / 2) / g.ngx
                               : (double)(i - g.nx - g.ny / 2) / g.ngy;
    double s = 0.0;
    for (int q = 0; q < quad.n; ++q) s += quad.w[q] * cos(2.0 * M_PI * quad.x[q] * nu);
    const double f = 1.0 / (2.0 * s);
    if (i < g.nx)
      cu[i] = f;
    else
      cv[i - g.nx] = f;
  }
}

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

static int fft_create(cufftHandle *h) {
  if (cufftCreate(h) != CUFFT_SUCCESS) {
    set_error("cufftCreate failed");
    return GB_ERR_CUFFT;
  }
  if (cufftSetAutoAllocation(*h, 0) != CUFFT_SUCCESS) {
    set_error("cufftSetAutoAllocation failed");
    return GB_ERR_CUFFT;
  }
  return GB_OK;
}

// Transforms of `planes` planes x NP pols, batched: 2-D plans, or in column
// mode 1-D transforms of every row (the column kernels do the rest).
// (Pruning to the image's columns through 1-D strided cuFFT plans measured
// slower on GB300 than the batched 2-D plan; the column kernels replace
// those strided plans.)
static int make_fft(gb_plan *p, int planes, cufftHandle *h, size_t *work) {
  const Geom &g = p->g;
  int rc = fft_create(h);
  if (rc) return rc;
  const cufftType type = p->precision == GB_FP64 ? CUFFT_Z2Z : CUFFT_C2C;
  cufftResult r;
  long long n[2] = {g.ngy, g.ngx};
  long long batch = (long long)planes * g.NP;
  if (p->col_fft) {
    long long nr[1] = {g.ngx};
    batch *= g.ngy;
    r = cufftMakePlanMany64(*h, 1, nr, nullptr, 1, 0, nullptr, 1, 0, type, batch, work);
  } else {
    r = cufftMakePlanMany64(*h, 2, n, nullptr, 1, 0, nullptr, 1, 0, type, batch, work);
  }
  if (r != CUFFT_SUCCESS) {
    set_error("cufftMakePlanMany64 failed (%d) for %lld x %lld x %lld (%s)", (int)r, n[0],
              n[1], batch, p->col_fft ? "rows" : "2-D");
    return GB_ERR_CUFFT;
  }
  return GB_OK;
}

// Column mode applies to the FP32 form with a power-of-two grid height.
static int choose_fft_mode(gb_plan *p) {
  int n1, n2;
  const bool fits = p->precision == GB_FP32 && p->g.ngy == 2 * p->g.ny &&
                    (p->g.ngx - p->g.nx) % 4 == 0 && column_split(p->g.ngy, n1, n2);
  switch (p->params.fft_mode) {
    case GB_FFT_AUTO: p->col_fft = fits; break;
    case GB_FFT_CUFFT_2D: p->col_fft = false; break;
    case GB_FFT_COLUMNS:
      if (!fits) {
        set_error("fft_mode GB_FFT_COLUMNS needs the FP32 form, a grid height of twice the "
                  "image height, a power of two in [256, 32768], and an even column offset "
                  "(grid %d x %d, image %d x %d)", p->g.ngx, p->g.ngy, p->g.nx, p->g.ny);
        return GB_ERR_INVALID_ARG;
      }
      p->col_fft = true;
      break;
    default:
      set_error("unknown fft_mode %d", p->params.fft_mode);
      return GB_ERR_INVALID_ARG;
  }
  p->row_fft = p->col_fft && row_kernel_fits(p->g.ngx);
  return GB_OK;
}

static int layout_workspace(gb_plan *p) {
  const Geom &g = p->g;
  const size_t item_bytes = p->precision == GB_FP64 ? sizeof(ItemD) : sizeof(ItemF);
  const size_t cb = cplx_bytes(p->precision), rb = real_bytes(p->precision);
  const int64_t nb1 = g.nbuckets + 1;
  p->max_chunks = (size_t)g.nitems / kChunkItems +
                  (size_t)std::min<int64_t>(g.nbuckets, (int64_t)g.nitems) + 1;
  p->nbatches = (g.nplanes + g.B - 1) / g.B;
  size_t off = 0;
  p->off_items = off;
  off = align_up(off + item_bytes * (size_t)g.nitems);
  p->off_chunk_off = off;
  off = align_up(off + 4 * (size_t)nb1);
  p->off_chunks = off;
  off = align_up(off + sizeof(Chunk) * p->max_chunks);
  p->off_corr = off;
  off = align_up(off + rb * (size_t)g.nx * g.ny);
  p->off_tprime = off;
  off = align_up(off + (g.do_w ? 8 * (size_t)g.nx * g.ny : 0));
  p->off_screen = off;
  off = align_up(off + (p->col_fft && g.do_w ? 16 * (size_t)g.nx * g.ny : 0));
  p->off_twn = off;
  off = align_up(off + (p->col_fft ? 8 * (size_t)g.ngy : 0));
  p->off_twx = off;
  off = align_up(off + (p->row_fft ? 8 * (size_t)g.ngx : 0));
  p->off_rowmask = off;
  off = align_up(off + (p->col_fft ? (size_t)g.nplanes * g.ntv : 0));
  p->off_tables = off;
  off = align_up(off + 8 * ((size_t)g.nx + g.ny + 2 * kMaxQuad));
  // shifted plans keep uvw and f/c: a PSF call rebuilds the unshifted factor
  p->off_coords = off;
  off = align_up(off + (g.shifted ? 8 * (3 * (size_t)g.R + g.C) : 0));
  p->off_counters = off;
  off = align_up(off + 4 * (size_t)(2 * p->nbatches + 8));
  p->off_fftwork = off;
  off = align_up(off + p->fft_work_bytes);
  p->off_temp = off;
  // bind temporaries
  size_t t = 0;
  p->t_keys = t;
  t = align_up(t + 4 * (size_t)g.nitems);
  p->t_ranks = t;
  t = align_up(t + 4 * (size_t)g.nitems);
  const int64_t nk1 = g.nbuckets * g.S + 1;  // sort keys (+ the end)
  p->t_counts = t;
  t = align_up(t + 4 * (size_t)nk1);
  p->t_offsets = t;
  t = align_up(t + 4 * (size_t)nk1);
  p->t_ccounts = t;
  t = align_up(t + 4 * (size_t)nb1);
  p->t_scan = t;
  t = align_up(t + 4 * scan_tmp_words(nk1));
  p->t_fscale = t;
  t = align_up(t + 8 * (size_t)g.C);
  const size_t bind_temp = t;
  // call temporaries
  size_t c = 0;
  p->c_grid = c;
  c = align_up(c + cb * (size_t)g.B * g.NP * g.ngx * (size_t)g.ngy);
  p->c_img = c;
  c = align_up(c + rb * (size_t)g.NP * g.nx * (size_t)g.ny);
  p->c_cvis = c;
  c = align_up(c + cb * (size_t)g.NP * g.nitems);
  const size_t call_temp = c;
  p->ws_bytes = off + std::max(bind_temp, call_temp);
  return GB_OK;
}

template <typename R>
static int run_bind(gb_plan *p, cudaStream_t s) {
  using Item = typename Traits<R>::Item;
  const Geom &g = p->g;
  char *tmp = p->ws + p->off_temp;
  uint32_t *keys = reinterpret_cast<uint32_t *>(tmp + p->t_keys);
  uint32_t *ranks = reinterpret_cast<uint32_t *>(tmp + p->t_ranks);
  uint32_t *counts = reinterpret_cast<uint32_t *>(tmp + p->t_counts);
  uint32_t *offsets = reinterpret_cast<uint32_t *>(tmp + p->t_offsets);
  uint32_t *ccounts = reinterpret_cast<uint32_t *>(tmp + p->t_ccounts);
  uint32_t *stmp = reinterpret_cast<uint32_t *>(tmp + p->t_scan);
  Item *items = p->at<Item>(p->off_items);
  uint32_t *chunk_off = p->at<uint32_t>(p->off_chunk_off);
  Chunk *chunks = p->at<Chunk>(p->off_chunks);
  const int64_t nb = g.nbuckets;
  const unsigned item_blocks =
      (unsigned)std::min<int64_t>(((int64_t)g.nitems + kThreads - 1) / kThreads,
                                  (int64_t)p->num_sms * 16);
  const unsigned bucket_blocks = (unsigned)std::min<int64_t>(
      (nb + kThreads - 1) / kThreads, (int64_t)p->num_sms * 16);
  const double ni = (double)g.nitems, rows = (double)g.R * 24.0 + 8.0 * g.C;
  const int64_t nk = nb * g.S;  // sort keys
  GB_CUDA(cudaMemsetAsync(counts, 0, 4 * (size_t)(nk + 1), s));
  GB_CUDA(cudaMemsetAsync(p->status_word(), 0, 4, s));
  double *fscale = reinterpret_cast<double *>(tmp + p->t_fscale);
  k_freq_scale<<<(g.C + kThreads - 1) / kThreads, kThreads, 0, s>>>(p->freq, g.C, fscale);
  GB_LAUNCH_CHECK("k_freq_scale");
  if (g.shifted) {
    GB_CUDA(cudaMemcpyAsync(p->at<double>(p->off_coords), p->uvw, 24 * (size_t)g.R,
                            cudaMemcpyDeviceToDevice, s));
    GB_CUDA(cudaMemcpyAsync(p->at<double>(p->off_coords) + 3 * (size_t)g.R, fscale,
                            8 * (size_t)g.C, cudaMemcpyDeviceToDevice, s));
  }
  {
    ProfScope ps(kProfCountKernel, s, rows + 8.0 * ni);
    k_count<<<item_blocks, kThreads, 0, s>>>(g, p->uvw, fscale, counts, keys, ranks);
    GB_LAUNCH_CHECK("k_count");
  }
  int rc;
  {
    ProfScope ps(kProfScan, s, 8.0 * (double)(nk + 1));
    rc = scan_exclusive(counts, offsets, nk, stmp, s);
  }
  if (rc) return rc;
  {
    ProfScope ps(kProfScatter, s, rows + ni * (12.0 + sizeof(Item)));
    k_scatter<R><<<item_blocks, kThreads, 0, s>>>(g, p->uvw, fscale, keys, ranks, offsets,
                                                   items);
    GB_LAUNCH_CHECK("k_scatter");
  }
  {
    ProfScope ps(kProfChunks, s, 20.0 * (double)(nb + 1) + 16.0 * ni / kChunkItems);
    k_chunk_counts<<<bucket_blocks, kThreads, 0, s>>>(offsets, g.S, nb, ccounts);
    GB_LAUNCH_CHECK("k_chunk_counts");
    rc = scan_exclusive(ccounts, chunk_off, nb, stmp, s);
    if (rc) return rc;
    k_emit_chunks<<<bucket_blocks, kThreads, 0, s>>>(offsets, g.S, chunk_off, nb, chunks);
    GB_LAUNCH_CHECK("k_emit_chunks");
  }
  // first item of every slab, to the host: only the profiler's byte counts
  // use it, and it costs a synchronisation, so only while profiling is on
  if (prof_on()) {
    uint32_t *slab_dev = ccounts;  // reuse: ccounts is free after the chunk scan
    k_slab_items<<<4, kThreads, 0, s>>>(offsets, g.nslabs, (int64_t)g.ntu * g.ntv, g.S,
                                        slab_dev);
    GB_LAUNCH_CHECK("k_slab_items");
    p->slab_items.assign((size_t)g.nslabs + 1, 0u);
    GB_CUDA(cudaMemcpyAsync(p->slab_items.data(), slab_dev, 4 * ((size_t)g.nslabs + 1),
                            cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
  }
  // correction factors
  double *tables = p->at<double>(p->off_tables);
  double *cu = tables, *cv = tables + g.nx;
  k_corr_1d<<<(g.nx + g.ny + kThreads - 1) / kThreads, kThreads, 0, s>>>(g, p->quad, cu, cv);
  GB_LAUNCH_CHECK("k_corr_1d");
  const int64_t npix = (int64_t)g.nx * g.ny;
  const unsigned pix_blocks = (unsigned)std::min<int64_t>((npix + kThreads - 1) / kThreads,
                                                          (int64_t)p->num_sms * 32);
  {
    ProfScope ps(kProfCorr, s, (double)npix * (sizeof(R) + (g.do_w ? 8.0 : 0.0)));
    ulonglong2 *screen = p->col_fft && g.do_w ? p->at<ulonglong2>(p->off_screen) : nullptr;
    k_corr_image<R><<<pix_blocks, kThreads, 0, s>>>(g, cu, cv, p->quad, p->at<R>(p->off_corr),
                                                     p->at<double>(p->off_tprime), screen);
    GB_LAUNCH_CHECK("k_corr_image");
  }
  if (p->col_fft) {
    k_twiddles<<<(g.ngy + kThreads - 1) / kThreads, kThreads, 0, s>>>(g.ngy,
                                                                     p->at<float2>(p->off_twn));
    GB_LAUNCH_CHECK("k_twiddles");
  }
  if (p->row_fft) {
    k_twiddles<<<(g.ngx + kThreads - 1) / kThreads, kThreads, 0, s>>>(g.ngx,
                                                                     p->at<float2>(p->off_twx));
    GB_LAUNCH_CHECK("k_twiddles");
  }
  if (p->col_fft) {
    uint8_t *mask = p->at<uint8_t>(p->off_rowmask);
    GB_CUDA(cudaMemsetAsync(mask, 0, (size_t)g.nplanes * g.ntv, s));
    const unsigned cb = (unsigned)std::min<int64_t>(
        ((int64_t)p->max_chunks + kThreads - 1) / kThreads, (int64_t)p->num_sms * 16);
    k_row_mask<<<cb, kThreads, 0, s>>>(g, chunks, chunk_off, mask);
    GB_LAUNCH_CHECK("k_row_mask");
    if (prof_on()) {  // host copy for the profiler's byte counts (costs a sync)
      p->mask_host.assign((size_t)g.nplanes * g.ntv, 0);
      GB_CUDA(cudaMemcpyAsync(p->mask_host.data(), mask, p->mask_host.size(),
                              cudaMemcpyDeviceToHost, s));
      GB_CUDA(cudaStreamSynchronize(s));
    }
  }
  if (prof_on()) {
    const int rc2 = plane_stats<Item>(p, s);
    if (rc2) return rc2;
  }
  return GB_OK;
}


// Verification export: per original item, its bucket, first support cell
// (p0, q0, k0) and offsets (du, dv, dwf) as stored in bucket order.
template <typename R>
__global__ void k_export_items(const Geom g, const typename Traits<R>::Item *__restrict__ items,
                               const Chunk *__restrict__ chunks,
                               const uint32_t *__restrict__ chunk_off,
                               uint32_t *__restrict__ bucket_out, int32_t *__restrict__ cell_out,
                               double *__restrict__ frac_out) {
  const uint32_t nchunks = chunk_off[g.nbuckets];
  const int ntiles = g.ntu * g.ntv;
  for (uint32_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const int slab = (int)(ch.bucket / (uint32_t)ntiles);
    const int tile = (int)(ch.bucket - (uint32_t)slab * ntiles);
    const int tv = tile / g.ntu, tu = tile - tv * g.ntu;
    for (uint32_t pos = ch.begin + threadIdx.x; pos < ch.end; pos += blockDim.x) {
      const auto it = items[pos];
      const uint32_t i = it.idx;
      if (bucket_out) bucket_out[i] = ch.bucket;
      if (cell_out) {
        cell_out[3 * (size_t)i] = tu * g.T + (int)(it.loc & 0xffu);
        cell_out[3 * (size_t)i + 1] = tv * g.T + (int)((it.loc >> 8) & 0xffu);
        cell_out[3 * (size_t)i + 2] = slab * g.S + (int)((it.loc >> 16) & 0xffu);
      }
      if (frac_out) {
        frac_out[3 * (size_t)i] = (double)it.du;
        frac_out[3 * (size_t)i + 1] = (double)it.dv;
        frac_out[3 * (size_t)i + 2] = (double)it.dwf;
      }
    }
  }
}

}  // namespace gb

using namespace gb;

extern "C" {

const char *gb_last_error_string(void) { return gb::last_error(); }

const char *gb_version(void) { return "rascil_gb300 0.1.0 (sm_103a)"; }

int gb_plan_geometry(const gb_plan_params *params, double w_lo, double w_hi,
                     gb_plan_info *info) {
  Geom g;
  int rc = plan_geometry(params, w_lo, w_hi, g);
  if (rc) return rc;
  if (!info) {
    set_error("info_out is NULL");
    return GB_ERR_INVALID_ARG;
  }
  gb_plan tmp;
  tmp.g = g;
  tmp.params = *params;
  tmp.precision = params->precision;
  tmp.fft_work_bytes = 0;
  rc = choose_fft_mode(&tmp);
  if (rc) return rc;
  layout_workspace(&tmp);
  memset(info, 0, sizeof(*info));
  info->support = g.W;
  info->ngrid_x = g.ngx;
  info->ngrid_y = g.ngy;
  info->nplanes = g.nplanes;
  info->planes_per_batch = g.B;
  info->tile = g.T;
  info->slab = g.S;
  info->beta = g.beta;
  info->sigma = g.sigma;
  info->dw = g.dw;
  info->w_lo = g.w_lo;
  info->w_hi = g.w_hi;
  info->tc = g.tc;
  info->nitems = g.nitems;
  info->nbuckets = g.nbuckets;
  info->workspace_bytes = (int64_t)tmp.ws_bytes;
  info->fft_mode = tmp.col_fft ? GB_FFT_COLUMNS : GB_FFT_CUFFT_2D;
  info->own_rows = tmp.row_fft ? 1 : 0;
  return GB_OK;
}

int gb_plan_create(const gb_plan_params *params, const double *uvw_dev,
                   const double *freq_dev, void *stream, gb_plan **plan_out) {
  if (!params || !uvw_dev || !freq_dev || !plan_out) {
    set_error("gb_plan_create: NULL argument");
    return GB_ERR_INVALID_ARG;
  }
  *plan_out = nullptr;
  if (params->nrows <= 0 || params->nchan <= 0) {
    set_error("nrows and nchan must be positive");
    return GB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  // frequencies to the host (validation and the w range)
  std::vector<double> freq(params->nchan);
  GB_CUDA(cudaMemcpyAsync(freq.data(), freq_dev, 8 * (size_t)params->nchan,
                          cudaMemcpyDeviceToHost, s));
  double w_lo = 0.0, w_hi = 0.0;
  {
    const int blocks = 512;
    double *part = nullptr;
    GB_CUDA(cudaMallocAsync((void **)&part, 3 * 8 * blocks, s));
    cudaError_t le;
    {
      ProfScope ps(kProfWrange, s, 24.0 * (double)params->nrows);
      k_wrange<<<blocks, kThreads, 0, s>>>(uvw_dev, params->nrows,
                                           params->do_wstacking ? 1 : 0, part);
      le = cudaGetLastError();
    }
    std::vector<double> hp(3 * blocks);
    cudaError_t ce = cudaMemcpyAsync(hp.data(), part, 3 * 8 * blocks, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(part, s);
    if (le != cudaSuccess) return cuda_fail(le, "k_wrange");
    if (ce != cudaSuccess) return cuda_fail(ce, "w range copy");
    GB_CUDA(cudaStreamSynchronize(s));
    double rlo = INFINITY, rhi = -INFINITY, bad = 0.0;
    for (int b = 0; b < blocks; ++b) {
      rlo = std::fmin(rlo, hp[3 * b]);
      rhi = std::fmax(rhi, hp[3 * b + 1]);
      bad += hp[3 * b + 2];
    }
    if (bad > 0.0) {
      set_error("uvw holds %.0f rows with non-finite values", bad);
      return GB_ERR_INVALID_ARG;
    }
    w_lo = INFINITY;
    w_hi = -INFINITY;
    for (int c = 0; c < params->nchan; ++c) {
      if (!(freq[c] > 0.0) || !std::isfinite(freq[c])) {
        set_error("frequency %d is not positive and finite (%g)", c, freq[c]);
        return GB_ERR_INVALID_ARG;
      }
      const double sc = freq[c] / kSpeedOfLight;
      w_lo = std::fmin(w_lo, std::fmin(rlo * sc, rhi * sc));
      w_hi = std::fmax(w_hi, std::fmax(rlo * sc, rhi * sc));
    }
  }
  gb_plan *p = new gb_plan();
  p->params = *params;
  p->precision = params->precision;
  int rc = plan_geometry(params, w_lo, w_hi, p->g);
  if (rc) {
    delete p;
    return rc;
  }
  p->uvw = uvw_dev;
  p->freq = freq_dev;
  make_quadrature(p->g, p->quad);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, dev);
  // cuFFT plans (host-side; the work area comes from the workspace)
  size_t w_full = 0, w_rem = 0;
  rc = choose_fft_mode(p);
  if (rc) {
    gb_plan_destroy(p);
    return rc;
  }
  p->rem_planes = p->g.nplanes % p->g.B;
  if (!p->row_fft) {
    rc = make_fft(p, p->g.B, &p->fft_full, &w_full);
    if (rc) {
      gb_plan_destroy(p);
      return rc;
    }
    p->fft_full_ok = true;
  }
  if (p->rem_planes && !p->row_fft) {
    rc = make_fft(p, p->rem_planes, &p->fft_rem, &w_rem);
    if (rc) {
      gb_plan_destroy(p);
      return rc;
    }
    p->fft_rem_ok = true;
  }
  // cuFFT refuses a work area that aliases the data, even when it reports
  // needing none, so the work area always gets a region of its own.  The
  // two plans never run concurrently and share it.
  p->fft_work_bytes = std::max<size_t>(std::max(w_full, w_rem), 4096);
  layout_workspace(p);
  rc = setup_tile_kernels(p);
  if (!rc) rc = setup_col_kernels(p);
  if (!rc) rc = setup_row_kernels(p);
  if (rc) {
    gb_plan_destroy(p);
    return rc;
  }
  *plan_out = p;
  return GB_OK;
}

int gb_plan_workspace_size(const gb_plan *plan, size_t *bytes) {
  if (!plan || !bytes) {
    set_error("gb_plan_workspace_size: NULL argument");
    return GB_ERR_INVALID_ARG;
  }
  *bytes = plan->ws_bytes;
  return GB_OK;
}

int gb_plan_bind(gb_plan *p, void *workspace, size_t bytes, void *stream) {
  if (!p) {
    set_error("gb_plan_bind: NULL plan");
    return GB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (!workspace) {
    set_error("gb_plan_bind: NULL workspace");
    return GB_ERR_WORKSPACE;
  }
  if (bytes < p->ws_bytes) {
    set_error("workspace of %zu bytes is smaller than the %zu the plan needs", bytes,
              p->ws_bytes);
    return GB_ERR_WORKSPACE;
  }
  if (((uintptr_t)workspace) & 255) {
    set_error("workspace must be 256-byte aligned");
    return GB_ERR_WORKSPACE;
  }
  p->ws = (char *)workspace;
  void *fw = p->ws + p->off_fftwork;
  const bool ok[2] = {p->fft_full_ok, p->fft_rem_ok};
  const cufftHandle hs[2] = {p->fft_full, p->fft_rem};
  for (int i = 0; i < 2; ++i) {
    if (ok[i] && cufftSetWorkArea(hs[i], fw) != CUFFT_SUCCESS) {
      set_error("cufftSetWorkArea failed");
      return GB_ERR_CUFFT;
    }
  }
  const int rc = p->precision == GB_FP64 ? run_bind<double>(p, s) : run_bind<float>(p, s);
  if (rc) return rc;
  p->bound = true;
  p->last_stream = s;
  return GB_OK;
}

int gb_plan_info_get(const gb_plan *p, gb_plan_info *info) {
  if (!p || !info) {
    set_error("gb_plan_info_get: NULL argument");
    return GB_ERR_INVALID_ARG;
  }
  const Geom &g = p->g;
  memset(info, 0, sizeof(*info));
  info->support = g.W;
  info->ngrid_x = g.ngx;
  info->ngrid_y = g.ngy;
  info->nplanes = g.nplanes;
  info->planes_per_batch = g.B;
  info->tile = g.T;
  info->slab = g.S;
  info->beta = g.beta;
  info->sigma = g.sigma;
  info->dw = g.dw;
  info->w_lo = g.w_lo;
  info->w_hi = g.w_hi;
  info->tc = g.tc;
  info->nitems = g.nitems;
  info->nbuckets = g.nbuckets;
  info->workspace_bytes = (int64_t)p->ws_bytes;
  info->fft_mode = p->col_fft ? GB_FFT_COLUMNS : GB_FFT_CUFFT_2D;
  info->own_rows = p->row_fft ? 1 : 0;
  return GB_OK;
}

int gb_plan_export_items(const gb_plan *p, uint32_t *bucket_dev, int32_t *cell_dev,
                         double *frac_dev, void *stream) {
  if (!p) {
    set_error("gb_plan_export_items: NULL plan");
    return GB_ERR_INVALID_ARG;
  }
  if (!p->bound) {
    set_error("gb_plan_export_items: plan has no workspace (call gb_plan_bind)");
    return GB_ERR_NOT_BOUND;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)(p->num_sms * 8);
  if (p->precision == GB_FP64)
    k_export_items<double><<<blocks, kThreads, 0, s>>>(
        p->g, p->at<ItemD>(p->off_items), p->at<Chunk>(p->off_chunks),
        p->at<uint32_t>(p->off_chunk_off), bucket_dev, cell_dev, frac_dev);
  else
    k_export_items<float><<<blocks, kThreads, 0, s>>>(
        p->g, p->at<ItemF>(p->off_items), p->at<Chunk>(p->off_chunks),
        p->at<uint32_t>(p->off_chunk_off), bucket_dev, cell_dev, frac_dev);
  GB_LAUNCH_CHECK("k_export_items");
  return GB_OK;
}

int gb_plan_device_status(gb_plan *p, void *stream, int32_t *status_out) {
  if (!p || !status_out) {
    set_error("gb_plan_device_status: NULL argument");
    return GB_ERR_INVALID_ARG;
  }
  if (!p->bound) {
    set_error("gb_plan_device_status: plan is not bound");
    return GB_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t v = 0;
  GB_CUDA(cudaMemcpyAsync(&v, p->status_word(), 4, cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemsetAsync(p->status_word(), 0, 4, s));
  GB_CUDA(cudaStreamSynchronize(s));
  *status_out = (int32_t)v;
  return GB_OK;
}

int gb_plan_destroy(gb_plan *p) {
  if (!p) return GB_OK;
  if (p->last_stream || p->bound) cudaStreamSynchronize(p->last_stream);
  if (p->fft_full_ok) cufftDestroy(p->fft_full);
  if (p->fft_rem_ok) cufftDestroy(p->fft_rem);
  delete p;
  return GB_OK;
}

}  // extern "C"
