// Tangent-plane phase rotation of visibilities in place: RASCIL's
// phaserotate_visibility with tangent=True
// (rascil/processing_components/visibility/base.py:296-357) and its phasor
// calculate_blockvisibility_phasor (:1248-1264), as one pass over the
// visibilities on the GPU.
//
//   k_rotate   one thread per (row, channel): d = ((u, v, w) . s) f / c
//              turns, formed and reduced modulo one turn in FP64, then every
//              pol multiplied by exp(+-2 pi i d).  The row's dot product is
//              taken in metres and scaled by the channel's f / c (a shared
//              table): seven FP64 instructions per (row, channel) instead of
//              a division and a dozen products -- every warp-level FP64
//              instruction costs 16 cycles of an SM's FP64 pipe on this part.
//
// The imaging path does not call this: invert / predict fuse the same
// rotation into the plan's per-item factors (gb_plan_params.phase_shift).
#include "gb_plan.cuh"

namespace gb {

constexpr int kRotTableChan = 4096;  // channels whose f / c is tabulated per block

template <typename R>
__global__ void k_rotate(const double *__restrict__ uvw, const double *__restrict__ freq,
                         int64_t nrows, int nchan, int npol, double sl, double sm, double sn,
                         double sign, typename Traits<R>::C *__restrict__ vis) {
  extern __shared__ double s_k[];
  const bool table = nchan <= kRotTableChan;
  if (table) {
    for (int c = threadIdx.x; c < nchan; c += blockDim.x) s_k[c] = gb_div(freq[c], kSpeedOfLight);
    __syncthreads();
  }
  const int64_t n = nrows * nchan;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / nchan;
    const int c = (int)(i - r * nchan);
    const double k = table ? s_k[c] : gb_div(freq[c], kSpeedOfLight);
    const double dm = fma(uvw[3 * r], sl, fma(uvw[3 * r + 1], sm, uvw[3 * r + 2] * sn));
    double d = dm * k;
    d -= rint(d);
    R s, co;
    sincos_2pi((R)(sign * d), &s, &co);
    auto *x = vis + i * npol;
    for (int p = 0; p < npol; ++p) {
      const auto a = x[p];
      x[p].x = a.x * co - a.y * s;
      x[p].y = a.x * s + a.y * co;
    }
  }
}

}  // namespace gb

using namespace gb;

extern "C" int gb_phase_rotate(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                               int32_t nchan, int32_t npol, void *vis_dev, int32_t precision,
                               double s_l, double s_m, double s_n, int32_t inverse,
                               void *stream) {
  if (!uvw_dev || !freq_dev || !vis_dev) {
    set_error("gb_phase_rotate: NULL argument");
    return GB_ERR_INVALID_ARG;
  }
  if (nrows < 0 || nchan <= 0 || npol <= 0 || npol > 4) {
    set_error("gb_phase_rotate: bad shape (%lld rows, %d channels, %d pols)",
              (long long)nrows, (int)nchan, (int)npol);
    return GB_ERR_INVALID_ARG;
  }
  if (precision != GB_FP32 && precision != GB_FP64) {
    set_error("gb_phase_rotate: unknown precision %d", (int)precision);
    return GB_ERR_INVALID_ARG;
  }
  if (!std::isfinite(s_l) || !std::isfinite(s_m) || !std::isfinite(s_n)) {
    set_error("gb_phase_rotate: direction cosines must be finite");
    return GB_ERR_INVALID_ARG;
  }
  const int64_t n = nrows * (int64_t)nchan;
  if (n == 0) return GB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, nsm = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const unsigned blocks =
      (unsigned)std::min<int64_t>((n + kThreads - 1) / kThreads, (int64_t)nsm * 16);
  // forward: the reference multiplies by conj(phasor) = exp(+2 pi i d)
  const double sign = inverse ? -1.0 : 1.0;
  const double cb = precision == GB_FP64 ? 16.0 : 8.0;
  ProfScope ps(kProfRotate, s, 2.0 * cb * (double)n * npol + 24.0 * nrows);
  const size_t smem = nchan <= kRotTableChan ? sizeof(double) * (size_t)nchan : 0;
  if (precision == GB_FP64)
    k_rotate<double><<<blocks, kThreads, smem, s>>>(uvw_dev, freq_dev, nrows, nchan, npol, s_l,
                                                    s_m, s_n, sign,
                                                    reinterpret_cast<double2 *>(vis_dev));
  else
    k_rotate<float><<<blocks, kThreads, smem, s>>>(uvw_dev, freq_dev, nrows, nchan, npol, s_l,
                                                   s_m, s_n, sign,
                                                   reinterpret_cast<float2 *>(vis_dev));
  GB_LAUNCH_CHECK("k_rotate");
  return GB_OK;
}
