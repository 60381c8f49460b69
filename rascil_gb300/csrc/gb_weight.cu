// Imaging weights: RASCIL's weight_visibility
// (rascil/processing_components/imaging/weighting.py:27-48) on the GPU.
//
//   k_wgrid    every (row, channel): its cell on the image-sized uv grid
//              (griddata/operations.py:71-107 builds the grid's WCS,
//              griddata/gridding.py:68-175 maps u, v to the nearest cell),
//              stored for k_wapply; the flagged imaging weights of its pols
//              are added to the grid with FP64 atomics (gridding.py:260-306);
//   k_wsums    sum(G) and sum(G^2) over the grid (the robust factor:
//              sum(G) equals the sum of all flagged imaging weights);
//   k_wrecip   each cell's divisor inverted once, in place: 1 / G (uniform)
//              or 1 / (1 + f2 G) (robust), 0 where G <= 0;
//   k_wapply   the new imaging weight of every sample (gridding.py:332-425)
//              from its stored cell: two products per sample.
//
// The grid is [image channel][v][u][pol]: the pols of a cell share one
// 32-byte sector, so a sample's atomics and its gather touch one sector.
//
// The cell is computed in FP64 with every rounding step explicit, in the
// order ((u - 0) / cdelt_u + crpix) - 1 then round-half-to-even, so it is
// bit-identical to the CPU restatement (and to the reference's linear WCS).
#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

#include "gb_plan.cuh"

namespace gb {

struct WeightGeom {
  int64_t R;
  int C, P, nx, ny, nci;
  double cdu, cdv;      // uv grid cell size (wavelengths; u negative for RA)
  double rcdu, rcdv;    // their reciprocals
  double crpu, crpv;    // 1-based reference pixel
  const int *vis_to_im;
  int ftype;
};

// numpy.nan_to_num: NaN -> 0, +-inf -> +-DBL_MAX.  Tested on the exponent
// bits (integer instructions: every FP64 instruction costs a warp 16 cycles
// of the SM's FP64 pipe on this part, and these kernels are bound by it).
__device__ __forceinline__ double nan_to_num(double x) {
  const long long b = __double_as_longlong(x);
  if (((b >> 52) & 0x7ff) != 0x7ff) return x;
  if (b & 0xfffffffffffffLL) return 0.0;
  return b < 0 ? -DBL_MAX : DBL_MAX;
}

// Grid index rint((x / cd + crp) - 1), rounded half to even, equal to what
// that IEEE sequence gives, or INT_MIN past 2^20 cells (off any grid).  The
// fast form fma(x, 1 / cd, crp - 1) differs from the IEEE sequence by under
// 6e-10 for |t| < 2^20 (the reciprocal's rounding, one rounding here, three
// there), which can change the rounding only that close to a half-integer;
// within 4e-9 of one the IEEE sequence itself is taken.  Four FP64
// instructions on the common path instead of a division's dozen.
__device__ __forceinline__ int grid_index(double x, double cd, double rcd, double crp) {
  double t = fma(x, rcd, crp - 1.0);
  double n = rint(t);
  if (!(fabs(t) < 1048576.0) || fabs(t - n) > 0.5 - 4e-9) {
    t = gb_sub(gb_add(gb_div(x, cd), crp), 1.0);
    n = rint(t);
    if (!(fabs(n) < 1048576.0)) return INT_MIN;
  }
  return (int)n;
}

// Cell (pu, pv) of row r at k = f / c; false if it lies outside the grid.
__device__ __forceinline__ bool weight_cell(const WeightGeom &w, const double *__restrict__ uvw,
                                            double k, int64_t r, int &pu, int &pv) {
  const double u = nan_to_num(gb_mul(uvw[3 * r], k));
  const double v = nan_to_num(gb_mul(uvw[3 * r + 1], k));
  pu = grid_index(u, w.cdu, w.rcdu, w.crpu);
  pv = grid_index(v, w.cdv, w.rcdv, w.crpv);
  return pu >= 0 && pu < w.nx && pv >= 0 && pv < w.ny;
}

// Flag values other than 0 and 1, out of line: a predicated inline form
// would issue its FP64 conversion and product for every sample.
__device__ __noinline__ double flagged_general(double x, long long f) {
  return x * (double)(1 - f);
}

// x * (1 - flag), as the reference forms the flagged imaging weight, in
// integer instructions for flags 0 and 1: x * 1.0 == x; x * 0.0 is a zero
// of x's sign, or NaN for x infinite or NaN.
__device__ __forceinline__ double flagged(double x, const void *flags, int ftype, int64_t i) {
  long long f = 0;
  if (ftype == GB_FLAGS_I64) f = reinterpret_cast<const long long *>(flags)[i];
  else if (ftype == GB_FLAGS_U8) f = reinterpret_cast<const uint8_t *>(flags)[i];
  if (f == 0) return x;
  if (f != 1) return flagged_general(x, f);
  const long long b = __double_as_longlong(x);
  const bool finite = ((b >> 52) & 0x7ff) != 0x7ff;
  return __longlong_as_double(finite ? (b & (long long)0x8000000000000000ULL)
                                     : 0x7ff8000000000000LL);
}

constexpr uint32_t kNoCell = 0xffffffffu;
// channels whose f / c k_wgrid tabulates in shared memory (else per sample)
constexpr int kMaxTableChan = 4096;

// 1 / g for g > 0 by Newton-Raphson (r <- r + r (1 - g r), twice) from the
// FP32 reciprocal: the relative error squares each step, 2^-23 -> 2^-46 ->
// below FP64 rounding, in four FMAs instead of an IEEE FP64 division (FP64
// runs at 1/64 of the FP32 rate on this part).  g outside FP32's normal
// range takes the division.
__device__ __forceinline__ double recip_pos(double g) {
  const float gf = (float)g;
  if (!(gf >= FLT_MIN && gf <= 0.5f * FLT_MAX)) return 1.0 / g;
  double r = (double)__frcp_rn(gf);
  r = fma(r, fma(-g, r, 1.0), r);
  r = fma(r, fma(-g, r, 1.0), r);
  return r;
}

__global__ void k_wgrid(const WeightGeom w, const double *__restrict__ uvw,
                        const double *__restrict__ freq, const double *__restrict__ imw,
                        const void *__restrict__ flags, double *__restrict__ grid,
                        uint32_t *__restrict__ cells, uint32_t *__restrict__ status) {
  extern __shared__ double s_k[];  // f / c per channel (C <= kMaxTableChan)
  const bool table = w.C <= kMaxTableChan;
  if (table) {
    for (int c = threadIdx.x; c < w.C; c += blockDim.x) s_k[c] = gb_div(freq[c], kSpeedOfLight);
    __syncthreads();
  }
  const int64_t n = w.R * w.C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / w.C;
    const int c = (int)(i - r * w.C);
    const double k = table ? s_k[c] : gb_div(freq[c], kSpeedOfLight);
    int pu, pv;
    if (!weight_cell(w, uvw, k, r, pu, pv)) {
      cells[i] = kNoCell;
      atomicOr(status, 1u);
      continue;
    }
    const uint32_t cell = (uint32_t)pv * (uint32_t)w.nx + (uint32_t)pu;
    cells[i] = cell;
    double *g = grid + ((int64_t)w.vis_to_im[c] * w.ny * w.nx + cell) * w.P;
    for (int p = 0; p < w.P; ++p) {
      const int64_t j = i * w.P + p;
      atomicAdd(&g[p], flagged(imw[j], flags, w.ftype, j));
    }
  }
}

__global__ void k_wsums(const double *__restrict__ grid, int64_t n, double *__restrict__ sums) {
  double s = 0.0, s2 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double g = grid[i];
    s += g;
    s2 += g * g;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  __shared__ double red[2][kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = s;
    red[1][warp] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < kWarps; ++k) {
      a += red[0][k];
      b += red[1][k];
    }
    atomicAdd(&sums[0], a);
    atomicAdd(&sums[1], b);
  }
}

__global__ void k_wrecip(double *__restrict__ grid, int64_t n, const double *__restrict__ sums,
                         int scheme, double a2) {
  // robust: f2 = (5 10^-R)^2 sum(w) / sum(G^2), with a2 = (5 10^-R)^2 from the host
  const double f2 = scheme == GB_WEIGHT_ROBUST ? a2 * sums[0] / sums[1] : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double g = grid[i];
    if (g > 0.0) grid[i] = recip_pos(scheme == GB_WEIGHT_ROBUST ? 1.0 + f2 * g : g);
    else if (g != 0.0) grid[i] = 0.0;
  }
}

__global__ void k_wapply(const WeightGeom w, const uint32_t *__restrict__ cells,
                         const double *__restrict__ imw, const double *__restrict__ wgt,
                         const void *__restrict__ flags, const double *__restrict__ grid,
                         const double *__restrict__ sums, int scheme, double a2,
                         double *__restrict__ out) {
  const int64_t n = w.R * w.C;
  const double f2 = scheme == GB_WEIGHT_ROBUST ? a2 * sums[0] / sums[1] : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (scheme == GB_WEIGHT_NATURAL) {
      for (int p = 0; p < w.P; ++p) out[i * w.P + p] = wgt[i * w.P + p];
      continue;
    }
    const int c = (int)(i % w.C);
    const uint32_t cell = cells[i];  // kNoCell: off the grid, already reported
    const double *gp =
        grid + (cell != kNoCell ? ((int64_t)w.vis_to_im[c] * w.ny * w.nx + cell) * w.P : 0);
    for (int p = 0; p < w.P; ++p) {
      const int64_t j = i * w.P + p;
      const double x = flagged(imw[j], flags, w.ftype, j);
      // the cell's inverted divisor (k_wrecip); positive exactly where G > 0
      const double rg = cell != kNoCell ? gp[p] : 0.0;
      double y = 0.0;
      if (__double_as_longlong(rg) > 0)  // rg is a positive double or +0
        y = scheme == GB_WEIGHT_UNIFORM ? x * (x * rg) : x * ((1.0 + f2 * x) * rg);
      out[j] = y;
    }
  }
}

}  // namespace gb

using namespace gb;

extern "C" int gb_weight_visibility(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                                    int32_t nchan, int32_t npol, const int32_t *vis_to_im_dev,
                                    int32_t nchan_img, int32_t nx, int32_t ny,
                                    double cdelt_x_deg, double cdelt_y_deg,
                                    const double *weight_dev, const double *imaging_weight_dev,
                                    const void *flags_dev, int32_t flags_type, int32_t weighting,
                                    double robustness, double *grid_dev, uint32_t *cells_dev,
                                    double *imaging_weight_out_dev, double *sums_dev,
                                    void *stream) {
  if (!uvw_dev || !freq_dev || !vis_to_im_dev || !weight_dev || !imaging_weight_dev ||
      !grid_dev || !cells_dev || !imaging_weight_out_dev || !sums_dev) {
    set_error("gb_weight_visibility: NULL argument");
    return GB_ERR_INVALID_ARG;
  }
  if (nrows <= 0 || nchan <= 0 || npol <= 0 || nchan_img <= 0 || nx <= 0 || ny <= 0 ||
      (int64_t)nx * ny >= (int64_t)kNoCell ||
      !(cdelt_x_deg != 0.0) || !(cdelt_y_deg != 0.0)) {
    set_error("gb_weight_visibility: empty or invalid geometry");
    return GB_ERR_INVALID_ARG;
  }
  if (weighting != GB_WEIGHT_NATURAL && weighting != GB_WEIGHT_UNIFORM &&
      weighting != GB_WEIGHT_ROBUST) {
    set_error("Weighting %d not supported", (int)weighting);
    return GB_ERR_INVALID_ARG;
  }
  if (flags_type != GB_FLAGS_NONE && flags_type != GB_FLAGS_U8 && flags_type != GB_FLAGS_I64) {
    set_error("gb_weight_visibility: unknown flags type %d", (int)flags_type);
    return GB_ERR_INVALID_ARG;
  }
  if (flags_type != GB_FLAGS_NONE && !flags_dev) {
    set_error("gb_weight_visibility: flags type given without flags");
    return GB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  // every channel must map to an image channel: the kernels index the grid
  // with it (the reference's numpy indexing raises for the same input)
  {
    std::vector<int32_t> v2i((size_t)nchan);
    GB_CUDA(cudaMemcpyAsync(v2i.data(), vis_to_im_dev, sizeof(int32_t) * (size_t)nchan,
                            cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    for (int32_t c = 0; c < nchan; ++c) {
      if (v2i[c] < 0 || v2i[c] >= nchan_img) {
        set_error("gb_weight_visibility: channel %d maps to image channel %d, outside [0, %d)",
                  (int)c, (int)v2i[c], (int)nchan_img);
        return GB_ERR_INVALID_ARG;
      }
    }
  }
  const double d2r = M_PI / 180.0;
  WeightGeom w;
  w.R = nrows;
  w.C = nchan;
  w.P = npol;
  w.nx = nx;
  w.ny = ny;
  w.nci = nchan_img;
  w.cdu = 1.0 / (nx * cdelt_x_deg * d2r);
  w.cdv = 1.0 / (ny * cdelt_y_deg * d2r);
  w.rcdu = 1.0 / w.cdu;
  w.rcdv = 1.0 / w.cdv;
  w.crpu = (double)(nx / 2 + 1);
  w.crpv = (double)(ny / 2 + 1);
  w.vis_to_im = vis_to_im_dev;
  w.ftype = flags_type;
  const int64_t ngrid = (int64_t)nchan_img * npol * ny * nx;
  int dev = 0, nsm = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  uint32_t *status = nullptr;
  GB_CUDA(cudaMallocAsync((void **)&status, sizeof(uint32_t), s));
  GB_CUDA(cudaMemsetAsync(status, 0, sizeof(uint32_t), s));
  GB_CUDA(cudaMemsetAsync(grid_dev, 0, sizeof(double) * (size_t)ngrid, s));
  GB_CUDA(cudaMemsetAsync(sums_dev, 0, 2 * sizeof(double), s));
  const int64_t n = nrows * (int64_t)nchan;
  const unsigned blocks =
      (unsigned)std::min<int64_t>((n + kThreads - 1) / kThreads, (int64_t)nsm * 16);
  // algorithmic bytes: per sample its imaging weight and flag (and weight /
  // new weight in the apply), per row its uvw; the grid once per pass
  const double fb = flags_type == GB_FLAGS_I64 ? 8.0 : (flags_type == GB_FLAGS_U8 ? 1.0 : 0.0);
  const double ns = (double)n * npol;
  {
    ProfScope ps(kProfWeightGrid, s, ns * (8.0 + fb) + 4.0 * n + 24.0 * nrows + 8.0 * ngrid);
    const size_t smem = nchan <= kMaxTableChan ? sizeof(double) * (size_t)nchan : 0;
    k_wgrid<<<blocks, kThreads, smem, s>>>(w, uvw_dev, freq_dev, imaging_weight_dev, flags_dev,
                                           grid_dev, cells_dev, status);
    GB_LAUNCH_CHECK("k_wgrid");
  }
  const unsigned gblocks =
      (unsigned)std::min<int64_t>((ngrid + kThreads - 1) / kThreads, (int64_t)nsm * 8);
  {
    ProfScope ps(kProfWeightSums, s, 8.0 * ngrid);
    k_wsums<<<gblocks, kThreads, 0, s>>>(grid_dev, ngrid, sums_dev);
    GB_LAUNCH_CHECK("k_wsums");
  }
  const double a = 5.0 * std::pow(10.0, -robustness);
  if (weighting != GB_WEIGHT_NATURAL) {
    ProfScope ps(kProfWeightRecip, s, 16.0 * ngrid);
    k_wrecip<<<gblocks, kThreads, 0, s>>>(grid_dev, ngrid, sums_dev, weighting, a * a);
    GB_LAUNCH_CHECK("k_wrecip");
  }
  {
    // uniform / robust: imaging weight, flag, inverted divisor in, new weight
    // out; per (row, channel) its cell
    const double per = weighting == GB_WEIGHT_NATURAL ? 16.0 : 24.0 + fb;
    ProfScope ps(kProfWeightApply, s,
                 ns * per + (weighting == GB_WEIGHT_NATURAL ? 0.0 : 4.0 * n));
    k_wapply<<<blocks, kThreads, 0, s>>>(w, cells_dev, imaging_weight_dev, weight_dev, flags_dev,
                                         grid_dev, sums_dev, weighting, a * a,
                                         imaging_weight_out_dev);
    GB_LAUNCH_CHECK("k_wapply");
  }
  uint32_t hs = 0;
  GB_CUDA(cudaMemcpyAsync(&hs, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaFreeAsync(status, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (hs) {
    set_error("a visibility's uv cell lies outside the %d x %d weighting grid (cellsize too "
              "large for the uv coverage)", nx, ny);
    return GB_ERR_OUT_OF_GRID;
  }
  return GB_OK;
}
