// Direct Fourier transforms on the GPU.
//
// k_dft_components  V[r][c][p] = sum_k flux[k][c][p] exp(-2 pi i uvw_lambda . (l, m, n-1))
//                   -- the reference's component DFT
//                   (rascil/processing_components/imaging/dft.py:123-178, CUDA
//                   kernel :181-258, CPU loop :261-281).  One thread per
//                   (row, channel) item; components staged through shared
//                   memory in tiles; the phase is accumulated in FP64 and
//                   reduced to [-1/2, 1/2] turns before the sincos.
// k_dft_pixels      exact dirty-image values at a list of pixels in ducc0's
//                   ms2dirty convention (the quantity the gridder
//                   approximates): sum Re(wgt V exp(+2 pi i f/c (x u + y v
//                   - w (n-1)))) / n.  One thread per pixel, visibilities
//                   staged through shared memory, FP64 partial sums added
//                   atomically per block.
// `exact` selects FP64 sincos; otherwise the reduced phase goes through the
// FP32 sincos (still FP64 phase arithmetic and FP64 accumulation).
#include <cmath>
#include <vector>

#include "gb_plan.cuh"

namespace gb {

constexpr int kDftTile = 128;

template <typename OutC>
__device__ __forceinline__ void store_c(OutC *p, double re, double im);
template <>
__device__ __forceinline__ void store_c<float2>(float2 *p, double re, double im) {
  *p = make_float2((float)re, (float)im);
}
template <>
__device__ __forceinline__ void store_c<double2>(double2 *p, double re, double im) {
  *p = make_double2(re, im);
}

__device__ __forceinline__ void turns_sincos(double turns, bool exact, double &s, double &c) {
  turns -= rint(turns);
  if (exact) {
    sincospi(2.0 * turns, &s, &c);
  } else {
    float fs, fc;
    sincospif(2.0f * (float)turns, &fs, &fc);
    s = fs;
    c = fc;
  }
}

template <typename OutC, int P>
__global__ void __launch_bounds__(kThreads)
    k_dft_components(const double *__restrict__ uvw, const double *__restrict__ freq,
                     int64_t nrows, int nchan, const double *__restrict__ lmn,
                     const double2 *__restrict__ flux, int ncomp, OutC *__restrict__ vis,
                     int exact) {
  __shared__ double s_lmn[kDftTile][3];
  const int64_t nitems = nrows * nchan;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nitems; base += stride) {
    const int64_t i = base + threadIdx.x;
    const bool active = i < nitems;
    const int64_t r = active ? i / nchan : 0;
    const int c = active ? (int)(i - r * nchan) : 0;
    const double s = freq[c] / kSpeedOfLight;
    const double u = uvw[3 * r] * s, v = uvw[3 * r + 1] * s, w = uvw[3 * r + 2] * s;
    double ar[P], ai[P];
#pragma unroll
    for (int p = 0; p < P; ++p) ar[p] = ai[p] = 0.0;
    for (int k0 = 0; k0 < ncomp; k0 += kDftTile) {
      const int nk = min(kDftTile, ncomp - k0);
      __syncthreads();
      for (int t = threadIdx.x; t < 3 * nk; t += blockDim.x) s_lmn[t / 3][t % 3] = lmn[3 * k0 + t];
      __syncthreads();
      if (active) {
        for (int k = 0; k < nk; ++k) {
          const double turns = u * s_lmn[k][0] + v * s_lmn[k][1] + w * s_lmn[k][2];
          double sn, cs;
          turns_sincos(turns, exact, sn, cs);
          // exp(-i theta) = cs - i sn
          const double2 *f = flux + ((size_t)(k0 + k) * nchan + c) * P;
#pragma unroll
          for (int p = 0; p < P; ++p) {
            const double2 fl = f[p];
            ar[p] += fl.x * cs + fl.y * sn;
            ai[p] += fl.y * cs - fl.x * sn;
          }
        }
      }
    }
    if (active) {
#pragma unroll
      for (int p = 0; p < P; ++p) store_c<OutC>(vis + i * P + p, ar[p], ai[p]);
    }
  }
}

// Uniformly spaced channels (f_c = f_0 + c df): for a row and a component the
// phase is linear in c, so exp(-2 pi i turns(c)) = base * step^c.  One thread
// per (row, block of CB channels) evaluates two FP64 sincospi per component
// and then one complex multiply per channel instead of a sincos; the
// recurrence adds about one rounding per channel (< 1e-14 relative over CB).
template <typename OutC, int P, int CB>
__global__ void __launch_bounds__(kThreads)
    k_dft_components_uniform(const double *__restrict__ uvw, double f0, double df,
                             int64_t nrows, int nchan, const double *__restrict__ lmn,
                             const double2 *__restrict__ flux, int ncomp,
                             OutC *__restrict__ vis) {
  __shared__ double s_lmn[kDftTile][3];
  const int c0 = blockIdx.y * CB;
  const int nc = min(CB, nchan - c0);
  const double s0 = (f0 + c0 * df) / kSpeedOfLight;
  const double ds = df / kSpeedOfLight;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nrows; base += stride) {
    const int64_t r = base + threadIdx.x;
    const bool active = r < nrows;
    const double u = active ? uvw[3 * r] : 0.0, v = active ? uvw[3 * r + 1] : 0.0,
                 w = active ? uvw[3 * r + 2] : 0.0;
    double ar[CB][P], ai[CB][P];
#pragma unroll
    for (int c = 0; c < CB; ++c)
#pragma unroll
      for (int p = 0; p < P; ++p) ar[c][p] = ai[c][p] = 0.0;
    for (int k0 = 0; k0 < ncomp; k0 += kDftTile) {
      const int nk = min(kDftTile, ncomp - k0);
      __syncthreads();
      for (int t = threadIdx.x; t < 3 * nk; t += blockDim.x) s_lmn[t / 3][t % 3] = lmn[3 * k0 + t];
      __syncthreads();
      if (!active) continue;
      for (int k = 0; k < nk; ++k) {
        const double d = u * s_lmn[k][0] + v * s_lmn[k][1] + w * s_lmn[k][2];
        double t0 = d * s0, dt = d * ds;
        t0 -= rint(t0);
        dt -= rint(dt);
        double bs, bc, ss, sc;
        sincospi(2.0 * t0, &bs, &bc);
        sincospi(2.0 * dt, &ss, &sc);
        double pr = bc, pi = -bs;         // exp(-2 pi i t0)
        const double qr = sc, qi = -ss;   // exp(-2 pi i dt)
        const double2 *f = flux + ((size_t)(k0 + k) * nchan + c0) * P;
#pragma unroll
        for (int c = 0; c < CB; ++c) {
          if (c < nc) {
#pragma unroll
            for (int p = 0; p < P; ++p) {
              const double2 fl = f[c * P + p];
              ar[c][p] += fl.x * pr - fl.y * pi;
              ai[c][p] += fl.x * pi + fl.y * pr;
            }
          }
          const double nr = pr * qr - pi * qi;
          pi = pr * qi + pi * qr;
          pr = nr;
        }
      }
    }
    if (active) {
#pragma unroll
      for (int c = 0; c < CB; ++c)
        if (c < nc)
#pragma unroll
          for (int p = 0; p < P; ++p)
            store_c<OutC>(vis + (((size_t)r * nchan + c0 + c) * P + p), ar[c][p], ai[c][p]);
    }
  }
}

template <typename InC, typename InR>
__global__ void __launch_bounds__(kThreads)
    k_dft_pixels(const double *__restrict__ uvw, const double *__restrict__ freq, int64_t nrows,
                 int nchan, int npol, int pol, const InC *__restrict__ ms,
                 const InR *__restrict__ wgt, const int32_t *__restrict__ pix, int npix, int nx,
                 int ny, double dx, double dy, int do_w, int exact, int64_t items_per_block,
                 double *__restrict__ out) {
  __shared__ double s_u[kThreads], s_v[kThreads], s_w[kThreads], s_re[kThreads],
      s_im[kThreads];
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  double x = 0.0, y = 0.0, t = 0.0;
  if (j < npix) {
    x = (double)(pix[2 * j] - nx / 2) * dx;
    y = (double)(pix[2 * j + 1] - ny / 2) * dy;
    if (do_w) {
      const double r2 = x * x + y * y;
      t = -r2 / (1.0 + sqrt(1.0 - r2));
    }
  }
  const int64_t nitems = nrows * nchan;
  const int64_t i0 = (int64_t)blockIdx.x * items_per_block;
  const int64_t i1 = min(nitems, i0 + items_per_block);
  double acc = 0.0;
  for (int64_t b = i0; b < i1; b += blockDim.x) {
    __syncthreads();
    const int64_t i = b + threadIdx.x;
    if (i < i1) {
      const int64_t r = i / nchan;
      const int c = (int)(i - r * nchan);
      const double s = freq[c] / kSpeedOfLight;
      s_u[threadIdx.x] = uvw[3 * r] * s;
      s_v[threadIdx.x] = uvw[3 * r + 1] * s;
      s_w[threadIdx.x] = uvw[3 * r + 2] * s;
      const InC m = ms[i * npol + pol];
      const double wt = wgt ? (double)wgt[i * npol + pol] : 1.0;
      s_re[threadIdx.x] = (double)m.x * wt;
      s_im[threadIdx.x] = (double)m.y * wt;
    } else {
      s_u[threadIdx.x] = s_v[threadIdx.x] = s_w[threadIdx.x] = 0.0;
      s_re[threadIdx.x] = s_im[threadIdx.x] = 0.0;
    }
    __syncthreads();
    if (j < npix) {
      const int n = (int)min((int64_t)blockDim.x, i1 - b);
      for (int k = 0; k < n; ++k) {
        const double turns = x * s_u[k] + y * s_v[k] - t * s_w[k];
        double sn, cs;
        turns_sincos(turns, exact, sn, cs);
        acc += s_re[k] * cs - s_im[k] * sn;
      }
    }
  }
  if (j < npix) atomicAdd(&out[j], acc / (1.0 + t));
}

}  // namespace gb

using namespace gb;

extern "C" {

int gb_dft_components(const double *uvw, const double *freq, int64_t nrows, int32_t nchan,
                      const double *lmn, const double *flux, int32_t ncomp, int32_t npol,
                      void *vis, int32_t vis_precision, int32_t exact, void *stream) {
  if (!uvw || !freq || !lmn || !flux || !vis || nrows <= 0 || nchan <= 0 || ncomp < 0) {
    set_error("gb_dft_components: invalid argument");
    return GB_ERR_INVALID_ARG;
  }
  if (npol != 1 && npol != 2 && npol != 4) {
    set_error("gb_dft_components: npol must be 1, 2 or 4");
    return GB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t nitems = nrows * (int64_t)nchan;
  const unsigned blocks =
      (unsigned)std::min<int64_t>((nitems + kThreads - 1) / kThreads, (int64_t)sms * 8);
  const double2 *f = reinterpret_cast<const double2 *>(flux);
  ProfScope ps(kProfDftComp, s,
               24.0 * nrows + (double)nitems * npol * (vis_precision == GB_FP64 ? 16.0 : 8.0));
  // exact FP64 on uniformly spaced channels: the channel-recurrence kernel
  bool uniform = false;
  double f0 = 0.0, df = 0.0;
  if (exact && nchan > 1) {
    std::vector<double> fh(nchan);
    GB_CUDA(cudaMemcpyAsync(fh.data(), freq, 8 * (size_t)nchan, cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    f0 = fh[0];
    df = (fh[nchan - 1] - fh[0]) / (nchan - 1);
    uniform = df != 0.0;
    for (int c = 0; c < nchan && uniform; ++c)
      uniform = std::fabs(fh[c] - (f0 + c * df)) <= 1e-13 * std::fabs(fh[c]);
  }
  if (uniform) {
    constexpr int CB4 = 4, CB8 = 8;
    const int cb = npol == 4 ? CB4 : CB8;
    const unsigned rblocks = (unsigned)std::min<int64_t>((nrows + kThreads - 1) / kThreads,
                                                         (int64_t)sms * 8);
    dim3 grid(rblocks, (unsigned)((nchan + cb - 1) / cb));
#define GB_DFTU(OutC, P, CB)                                                                  \
  k_dft_components_uniform<OutC, P, CB><<<grid, kThreads, 0, s>>>(                             \
      uvw, f0, df, nrows, nchan, lmn, f, ncomp, reinterpret_cast<OutC *>(vis))
    if (vis_precision == GB_FP64) {
      if (npol == 1) GB_DFTU(double2, 1, CB8);
      else if (npol == 2) GB_DFTU(double2, 2, CB8);
      else GB_DFTU(double2, 4, CB4);
    } else {
      if (npol == 1) GB_DFTU(float2, 1, CB8);
      else if (npol == 2) GB_DFTU(float2, 2, CB8);
      else GB_DFTU(float2, 4, CB4);
    }
#undef GB_DFTU
    GB_LAUNCH_CHECK("k_dft_components_uniform");
    return GB_OK;
  }
#define GB_DFT(OutC, P)                                                                   \
  k_dft_components<OutC, P><<<blocks, kThreads, 0, s>>>(uvw, freq, nrows, nchan, lmn, f,   \
                                                        ncomp, reinterpret_cast<OutC *>(vis), \
                                                        exact)
  if (vis_precision == GB_FP64) {
    if (npol == 1) GB_DFT(double2, 1);
    else if (npol == 2) GB_DFT(double2, 2);
    else GB_DFT(double2, 4);
  } else {
    if (npol == 1) GB_DFT(float2, 1);
    else if (npol == 2) GB_DFT(float2, 2);
    else GB_DFT(float2, 4);
  }
#undef GB_DFT
  GB_LAUNCH_CHECK("k_dft_components");
  return GB_OK;
}

int gb_dft_pixels(const double *uvw, const double *freq, int64_t nrows, int32_t nchan,
                  int32_t npol, int32_t pol, const void *ms, int32_t ms_precision,
                  const void *wgt, const int32_t *pix, int32_t npix, int32_t npix_x,
                  int32_t npix_y, double pixsize_x, double pixsize_y, int32_t do_wstacking,
                  int32_t exact, double *out, void *stream) {
  if (!uvw || !freq || !ms || !pix || !out || nrows <= 0 || nchan <= 0 || npix <= 0 ||
      pol < 0 || pol >= npol) {
    set_error("gb_dft_pixels: invalid argument");
    return GB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  GB_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)npix, s));
  const int64_t nitems = nrows * (int64_t)nchan;
  const int pix_groups = (npix + kThreads - 1) / kThreads;
  int64_t item_blocks = std::max<int64_t>(1, (int64_t)sms * 8 / pix_groups);
  int64_t per = (nitems + item_blocks - 1) / item_blocks;
  per = ((per + kThreads - 1) / kThreads) * kThreads;
  item_blocks = (nitems + per - 1) / per;
  dim3 grid((unsigned)item_blocks, (unsigned)pix_groups);
  ProfScope ps(kProfDftPix, s,
               24.0 * nrows + (double)nitems * (ms_precision == GB_FP64 ? 16.0 : 8.0));
  if (ms_precision == GB_FP64)
    k_dft_pixels<double2, double><<<grid, kThreads, 0, s>>>(
        uvw, freq, nrows, nchan, npol, pol, reinterpret_cast<const double2 *>(ms),
        reinterpret_cast<const double *>(wgt), pix, npix, npix_x, npix_y, pixsize_x, pixsize_y,
        do_wstacking, exact, per, out);
  else
    k_dft_pixels<float2, float><<<grid, kThreads, 0, s>>>(
        uvw, freq, nrows, nchan, npol, pol, reinterpret_cast<const float2 *>(ms),
        reinterpret_cast<const float *>(wgt), pix, npix, npix_x, npix_y, pixsize_x, pixsize_y,
        do_wstacking, exact, per, out);
  GB_LAUNCH_CHECK("k_dft_pixels");
  return GB_OK;
}

}  // extern "C"
