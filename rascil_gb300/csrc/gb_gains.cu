// Per-antenna complex gains for the differentiable predict.
//
// k_apply_gains     out[r][c][p] = g[a1(r)][c] conj(g[a2(r)][c]) vis[r][c][p]
// k_gain_gradient   for a real loss L of out, with G = dL/dRe(out) + i dL/dIm(out)
//                   (PyTorch's complex gradient), the gradient with respect to the
//                   gains is, per antenna i and channel c,
//                     sum_{r: a1(r)=i, p} g[a2][c] conj(vis) G
//                   + sum_{r: a2(r)=i, p} g[a1][c] vis conj(G).
//                   Each block accumulates its rows into a shared-memory table of
//                   all (antenna, channel) pairs when that fits, then adds the table
//                   to the output with one atomic per entry.
// Gains and their gradients are complex128; visibilities follow the precision.
#include "gb_plan.cuh"

namespace gb {

template <typename C> struct CTraits;
template <> struct CTraits<float2> { using R = float; };
template <> struct CTraits<double2> { using R = double; };

template <typename C>
__global__ void k_apply_gains(const C *__restrict__ vis, const double2 *__restrict__ gains,
                              const int32_t *__restrict__ a1, const int32_t *__restrict__ a2,
                              int64_t nrows, int nchan, int npol, C *__restrict__ out) {
  using R = typename CTraits<C>::R;
  const int64_t n = nrows * nchan;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t r = i / nchan;
    const int c = (int)(i - r * nchan);
    const double2 gi = gains[(size_t)a1[r] * nchan + c];
    const double2 gj = gains[(size_t)a2[r] * nchan + c];
    // gi * conj(gj)
    const double fr = gi.x * gj.x + gi.y * gj.y;
    const double fi = gi.y * gj.x - gi.x * gj.y;
    for (int p = 0; p < npol; ++p) {
      const C v = vis[i * npol + p];
      C o;
      o.x = (R)(fr * v.x - fi * v.y);
      o.y = (R)(fr * v.y + fi * v.x);
      out[i * npol + p] = o;
    }
  }
}

__device__ __forceinline__ void add_c(double2 *dst, double re, double im) {
  atomicAdd(&dst->x, re);
  atomicAdd(&dst->y, im);
}

template <typename C>
__global__ void k_gain_gradient(const C *__restrict__ vis, const C *__restrict__ grad,
                                const double2 *__restrict__ gains,
                                const int32_t *__restrict__ a1, const int32_t *__restrict__ a2,
                                int64_t nrows, int nchan, int npol, int nant, int use_smem,
                                double2 *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *tab = reinterpret_cast<double2 *>(smem_raw);
  const int ntab = nant * nchan;
  if (use_smem) {
    for (int t = threadIdx.x; t < ntab; t += blockDim.x) tab[t] = make_double2(0.0, 0.0);
    __syncthreads();
  }
  double2 *dst = use_smem ? tab : out;
  const int64_t n = nrows * nchan;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t r = i / nchan;
    const int c = (int)(i - r * nchan);
    const int i1 = a1[r], i2 = a2[r];
    const double2 g1 = gains[(size_t)i1 * nchan + c];
    const double2 g2 = gains[(size_t)i2 * nchan + c];
    // s1 = sum_p conj(V) G,  s2 = sum_p V conj(G)  (s2 = conj(s1))
    double sr = 0.0, si = 0.0;
    for (int p = 0; p < npol; ++p) {
      const C v = vis[i * npol + p];
      const C gg = grad[i * npol + p];
      sr += (double)v.x * gg.x + (double)v.y * gg.y;
      si += (double)v.x * gg.y - (double)v.y * gg.x;
    }
    // antenna a1: g2 * s1 ; antenna a2: g1 * conj(s1)
    add_c(&dst[(size_t)i1 * nchan + c], g2.x * sr - g2.y * si, g2.x * si + g2.y * sr);
    add_c(&dst[(size_t)i2 * nchan + c], g1.x * sr + g1.y * si, g1.y * sr - g1.x * si);
  }
  if (use_smem) {
    __syncthreads();
    for (int t = threadIdx.x; t < ntab; t += blockDim.x) {
      const double2 v = tab[t];
      if (v.x != 0.0 || v.y != 0.0) add_c(&out[t], v.x, v.y);
    }
  }
}

}  // namespace gb

using namespace gb;

static int check_gain_args(const void *vis, const double *gains, const int32_t *a1,
                           const int32_t *a2, int64_t nrows, int32_t nchan, int32_t npol,
                           int32_t precision) {
  if (!vis || !gains || !a1 || !a2 || nrows <= 0 || nchan <= 0 || npol < 1 || npol > 4 ||
      (precision != GB_FP32 && precision != GB_FP64)) {
    set_error("gain kernels: invalid argument");
    return GB_ERR_INVALID_ARG;
  }
  return GB_OK;
}

extern "C" {

int gb_apply_gains(const void *vis_dev, const double *gains_dev, const int32_t *ant1_dev,
                   const int32_t *ant2_dev, int64_t nrows, int32_t nchan, int32_t npol,
                   int32_t precision, void *out_dev, void *stream) {
  int rc = check_gain_args(vis_dev, gains_dev, ant1_dev, ant2_dev, nrows, nchan, npol, precision);
  if (rc) return rc;
  if (!out_dev) {
    set_error("gb_apply_gains: NULL output");
    return GB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t n = nrows * nchan;
  const unsigned blocks = (unsigned)std::min<int64_t>((n + kThreads - 1) / kThreads,
                                                      (int64_t)sms * 16);
  const double2 *g = reinterpret_cast<const double2 *>(gains_dev);
  if (precision == GB_FP64)
    k_apply_gains<double2><<<blocks, kThreads, 0, s>>>(
        reinterpret_cast<const double2 *>(vis_dev), g, ant1_dev, ant2_dev, nrows, nchan, npol,
        reinterpret_cast<double2 *>(out_dev));
  else
    k_apply_gains<float2><<<blocks, kThreads, 0, s>>>(
        reinterpret_cast<const float2 *>(vis_dev), g, ant1_dev, ant2_dev, nrows, nchan, npol,
        reinterpret_cast<float2 *>(out_dev));
  GB_LAUNCH_CHECK("k_apply_gains");
  return GB_OK;
}

int gb_gain_gradient(const void *vis_dev, const void *grad_dev, const double *gains_dev,
                     const int32_t *ant1_dev, const int32_t *ant2_dev, int64_t nrows,
                     int32_t nchan, int32_t npol, int32_t nant, int32_t precision,
                     double *grad_gains_dev, void *stream) {
  int rc = check_gain_args(vis_dev, gains_dev, ant1_dev, ant2_dev, nrows, nchan, npol, precision);
  if (rc) return rc;
  if (!grad_dev || !grad_gains_dev || nant <= 0) {
    set_error("gb_gain_gradient: invalid argument");
    return GB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t tab_bytes = sizeof(double2) * (size_t)nant * nchan;
  const int use_smem = tab_bytes <= 48 * 1024 ? 1 : 0;
  const int64_t n = nrows * nchan;
  const unsigned blocks = (unsigned)std::min<int64_t>((n + kThreads - 1) / kThreads,
                                                      (int64_t)sms * 4);
  double2 *out = reinterpret_cast<double2 *>(grad_gains_dev);
  const double2 *g = reinterpret_cast<const double2 *>(gains_dev);
  const size_t smem = use_smem ? tab_bytes : 0;
  if (precision == GB_FP64)
    k_gain_gradient<double2><<<blocks, kThreads, smem, s>>>(
        reinterpret_cast<const double2 *>(vis_dev), reinterpret_cast<const double2 *>(grad_dev),
        g, ant1_dev, ant2_dev, nrows, nchan, npol, nant, use_smem, out);
  else
    k_gain_gradient<float2><<<blocks, kThreads, smem, s>>>(
        reinterpret_cast<const float2 *>(vis_dev), reinterpret_cast<const float2 *>(grad_dev), g,
        ant1_dev, ant2_dev, nrows, nchan, npol, nant, use_smem, out);
  GB_LAUNCH_CHECK("k_gain_gradient");
  return GB_OK;
}

}  // extern "C"
