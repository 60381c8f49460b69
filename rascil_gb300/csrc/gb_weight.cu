// Imaging weights: RASCIL's weight_visibility
// (rascil/processing_components/imaging/weighting.py:27-48) on the GPU.
//
//   k_wgrid    every (row, channel): its cell on the image-sized uv grid
//              (griddata/operations.py:71-107 builds the grid's WCS,
//              griddata/gridding.py:68-175 maps u, v to the nearest cell);
//              the flagged imaging weights of its pols are added to the grid
//              with FP64 atomics (gridding.py:260-306);
//   k_wsums    sum(G) and sum(G^2) over the grid (the robust factor:
//              sum(G) equals the sum of all flagged imaging weights);
//   k_wapply   the new imaging weight of every sample (gridding.py:332-425).
//
// The cell is computed in FP64 with every rounding step explicit, in the
// order ((u - 0) / cdelt_u + crpix) - 1 then round-half-to-even, so it is
// bit-identical to the CPU restatement (and to the reference's linear WCS).
#include <cfloat>
#include <cmath>

#include "gb_plan.cuh"

namespace gb {

struct WeightGeom {
  int64_t R;
  int C, P, nx, ny, nci;
  double cdu, cdv;      // uv grid cell size (wavelengths; u negative for RA)
  double crpu, crpv;    // 1-based reference pixel
  const int *vis_to_im;
  int ftype;
};

__device__ __forceinline__ double nan_to_num(double x) {
  if (isnan(x)) return 0.0;
  if (isinf(x)) return x > 0 ? DBL_MAX : -DBL_MAX;
  return x;
}

// Cell (pu, pv) of row r, channel c; false if it lies outside the grid.
__device__ __forceinline__ bool weight_cell(const WeightGeom &w, const double *__restrict__ uvw,
                                            const double *__restrict__ freq, int64_t r, int c,
                                            int &pu, int &pv) {
  const double k = gb_div(freq[c], kSpeedOfLight);
  const double u = nan_to_num(gb_mul(uvw[3 * r], k));
  const double v = nan_to_num(gb_mul(uvw[3 * r + 1], k));
  const double xu = rint(gb_sub(gb_add(gb_div(u, w.cdu), w.crpu), 1.0));
  const double xv = rint(gb_sub(gb_add(gb_div(v, w.cdv), w.crpv), 1.0));
  if (!(xu >= 0.0 && xu < (double)w.nx && xv >= 0.0 && xv < (double)w.ny)) return false;
  pu = (int)xu;
  pv = (int)xv;
  return true;
}

__device__ __forceinline__ double flag_factor(const void *flags, int ftype, int64_t i) {
  if (ftype == GB_FLAGS_I64) return (double)(1 - reinterpret_cast<const long long *>(flags)[i]);
  if (ftype == GB_FLAGS_U8) return (double)(1 - (int)reinterpret_cast<const uint8_t *>(flags)[i]);
  return 1.0;
}

__global__ void k_wgrid(const WeightGeom w, const double *__restrict__ uvw,
                        const double *__restrict__ freq, const double *__restrict__ imw,
                        const void *__restrict__ flags, double *__restrict__ grid,
                        uint32_t *__restrict__ status) {
  const int64_t n = w.R * w.C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / w.C;
    const int c = (int)(i - r * w.C);
    int pu, pv;
    if (!weight_cell(w, uvw, freq, r, c, pu, pv)) {
      atomicOr(status, 1u);
      continue;
    }
    const int ic = w.vis_to_im[c];
    for (int p = 0; p < w.P; ++p) {
      const int64_t j = i * w.P + p;
      const double fw = imw[j] * flag_factor(flags, w.ftype, j);
      atomicAdd(&grid[(((int64_t)ic * w.P + p) * w.ny + pv) * w.nx + pu], fw);
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

__global__ void k_wapply(const WeightGeom w, const double *__restrict__ uvw,
                         const double *__restrict__ freq, const double *__restrict__ imw,
                         const double *__restrict__ wgt, const void *__restrict__ flags,
                         const double *__restrict__ grid, const double *__restrict__ sums,
                         int scheme, double a2, double *__restrict__ out) {
  const int64_t n = w.R * w.C;
  // robust: f2 = (5 10^-R)^2 sum(w) / sum(G^2), with a2 = (5 10^-R)^2 from the host
  const double f2 = scheme == GB_WEIGHT_ROBUST ? a2 * sums[0] / sums[1] : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (scheme == GB_WEIGHT_NATURAL) {
      for (int p = 0; p < w.P; ++p) out[i * w.P + p] = wgt[i * w.P + p];
      continue;
    }
    const int64_t r = i / w.C;
    const int c = (int)(i - r * w.C);
    int pu = 0, pv = 0;
    const bool in = weight_cell(w, uvw, freq, r, c, pu, pv);  // out-of-grid already reported
    const int ic = w.vis_to_im[c];
    for (int p = 0; p < w.P; ++p) {
      const int64_t j = i * w.P + p;
      const double x = imw[j] * flag_factor(flags, w.ftype, j);
      const double g = in ? grid[(((int64_t)ic * w.P + p) * w.ny + pv) * w.nx + pu] : 0.0;
      double y = 0.0;
      if (g > 0.0) {
        y = scheme == GB_WEIGHT_UNIFORM ? x * (x / g) : x * ((1.0 + f2 * x) / (1.0 + f2 * g));
      }
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
                                    double robustness, double *grid_dev,
                                    double *imaging_weight_out_dev, double *sums_dev,
                                    void *stream) {
  if (!uvw_dev || !freq_dev || !vis_to_im_dev || !weight_dev || !imaging_weight_dev ||
      !grid_dev || !imaging_weight_out_dev || !sums_dev) {
    set_error("gb_weight_visibility: NULL argument");
    return GB_ERR_INVALID_ARG;
  }
  if (nrows <= 0 || nchan <= 0 || npol <= 0 || nchan_img <= 0 || nx <= 0 || ny <= 0 ||
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
  k_wgrid<<<blocks, kThreads, 0, s>>>(w, uvw_dev, freq_dev, imaging_weight_dev, flags_dev,
                                      grid_dev, status);
  GB_LAUNCH_CHECK("k_wgrid");
  const unsigned gblocks =
      (unsigned)std::min<int64_t>((ngrid + kThreads - 1) / kThreads, (int64_t)nsm * 8);
  k_wsums<<<gblocks, kThreads, 0, s>>>(grid_dev, ngrid, sums_dev);
  GB_LAUNCH_CHECK("k_wsums");
  const double a = 5.0 * std::pow(10.0, -robustness);
  k_wapply<<<blocks, kThreads, 0, s>>>(w, uvw_dev, freq_dev, imaging_weight_dev, weight_dev,
                                       flags_dev, grid_dev, sums_dev, weighting, a * a,
                                       imaging_weight_out_dev);
  GB_LAUNCH_CHECK("k_wapply");
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
