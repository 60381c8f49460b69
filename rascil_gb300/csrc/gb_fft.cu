// Fused, pruned column transforms for power-of-two grid heights (FP32 form).
//
// A w-plane's 2-D transform is done as row transforms (batched 1-D cuFFT
// over contiguous rows) plus column transforms written here.  The image
// occupies only the nx central columns and ny central rows of each plane
// (checkerboarded grids), so only those columns are transformed, by a
// four-step split of the column length n = N1 N2 (q = N2 q1 + q2,
// k = k1 + N1 k2):
//
//   step A  for each q2: the N1-point DFT over q1 of x[N2 q1 + q2], times
//           exp(s 2 pi i q2 k1 / n), stored back at rows N2 k1 + q2;
//   step B  for each k1: the N2-point DFT over the contiguous rows
//           N2 k1 + q2 gives X[k1 + N1 k2].
//
// A CTA transforms a tile of kTC = 16 adjacent columns (128-byte row
// segments) with radix-8/4/2 Stockham passes in shared memory.  Fusions:
//
//   invert  (rows first, then columns)  step B never writes the plane back:
//           it keeps only the image rows, applies each plane's w-screen
//           exp(-2 pi i w_k (n-1-tc)) and accumulates the image in registers
//           over the batch's planes, so a batch costs one read-modify-write
//           of the image instead of a pass over every plane;
//   predict (columns first, then rows)  step A builds its input from the
//           corrected image (screen exp(+2 pi i w_k (n-1-tc)) on the image
//           rows, zero elsewhere) instead of reading a padded grid, and
//           step B writes in place, so physical row N2 k1 + k2 holds logical
//           row k1 + N1 k2; the degridder reads rows through that
//           permutation (RowPerm).
#include <cufft.h>

#include "gb_fft.cuh"

namespace gb {

constexpr int kTC = 16;  // columns per tile

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// a * (s i)
template <int S> __device__ __forceinline__ float2 mul_si(float2 a) {
  return S > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// In-register R-point DFTs, z_q = sum_p a_p exp(s 2 pi i p q / R).
template <int S> __device__ __forceinline__ void dft2(float2 *a) {
  const float2 t = a[0];
  a[0] = cadd(t, a[1]);
  a[1] = csub(t, a[1]);
}

template <int S> __device__ __forceinline__ void dft4(float2 *a) {
  const float2 s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
  const float2 s13 = cadd(a[1], a[3]), d13 = mul_si<S>(csub(a[1], a[3]));
  a[0] = cadd(s02, s13);
  a[2] = csub(s02, s13);
  a[1] = cadd(d02, d13);
  a[3] = csub(d02, d13);
}

template <int S> __device__ __forceinline__ void dft8(float2 *a) {
  float2 e[4] = {a[0], a[2], a[4], a[6]};
  float2 o[4] = {a[1], a[3], a[5], a[7]};
  dft4<S>(e);
  dft4<S>(o);
  const float r = 0.70710678118654752f;  // cos(pi/4)
  const float2 w1 = make_float2(r, S * r), w3 = make_float2(-r, S * r);
  const float2 t0 = o[0], t1 = cmul(o[1], w1), t2 = mul_si<S>(o[2]), t3 = cmul(o[3], w3);
  a[0] = cadd(e[0], t0);
  a[4] = csub(e[0], t0);
  a[1] = cadd(e[1], t1);
  a[5] = csub(e[1], t1);
  a[2] = cadd(e[2], t2);
  a[6] = csub(e[2], t2);
  a[3] = cadd(e[3], t3);
  a[7] = csub(e[3], t3);
}

template <int R, int S> __device__ __forceinline__ void dftR(float2 *a) {
  if (R == 2) dft2<S>(a);
  else if (R == 4) dft4<S>(a);
  else dft8<S>(a);
}

// One Stockham pass of radix R over the [L][kTC] tile in `x`, in place:
// every thread loads the inputs of its butterflies into registers, the
// block synchronises, and the outputs overwrite the same buffer.
// tw[m] = exp(s 2 pi i m / L).
template <int L, int R, int S>
__device__ __forceinline__ void stockham_pass(float2 *x, int Ls, const float2 *__restrict__ tw) {
  constexpr int NB = L / R;
  constexpr int NBF = NB * kTC;  // butterflies in the tile
  constexpr int BPT = (NBF + kThreads - 1) / kThreads;
  const int tstep = L / (Ls * R);
  float2 a[BPT][R];
#pragma unroll
  for (int t = 0; t < BPT; ++t) {
    const int b = threadIdx.x + t * kThreads;
    if (NBF % kThreads == 0 || b < NBF) {
      const int c = b % kTC, j = b / kTC;
      const int k = j & (Ls - 1);
#pragma unroll
      for (int p = 0; p < R; ++p) {
        a[t][p] = x[(j + p * NB) * kTC + c];
        if (p > 0) a[t][p] = cmul(a[t][p], tw[(p * k * tstep) & (L - 1)]);
      }
      dftR<R, S>(a[t]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < BPT; ++t) {
    const int b = threadIdx.x + t * kThreads;
    if (NBF % kThreads == 0 || b < NBF) {
      const int c = b % kTC, j = b / kTC;
      const int k = j & (Ls - 1);
      const int base = (j - k) * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) x[(base + q * Ls) * kTC + c] = a[t][q];
    }
  }
  __syncthreads();
}

// Natural-order L-point transform of every column of the tile, in place.
// Radix plan: as many radix-8 passes as fit, then one radix-4 or radix-2.
// The caller synchronises before (tile and twiddles written).
template <int L, int S>
__device__ __forceinline__ void tile_fft(float2 *x, const float2 *tw) {
  constexpr int lg = L == 256 ? 8 : L == 128 ? 7 : L == 64 ? 6 : L == 32 ? 5 : 4;
  static_assert((1 << lg) == L, "tile length must be 16..256");
  constexpr int e8 = lg / 3, rem = lg % 3;
  int Ls = 1;
#pragma unroll
  for (int i = 0; i < e8; ++i) {
    stockham_pass<L, 8, S>(x, Ls, tw);
    Ls *= 8;
  }
  if (rem == 2) stockham_pass<L, 4, S>(x, Ls, tw);
  if (rem == 1) stockham_pass<L, 2, S>(x, Ls, tw);
}

template <int L, int S>
__device__ __forceinline__ void make_twiddles(float2 *tw) {
  for (int m = threadIdx.x; m < L; m += blockDim.x) {
    float s, c;
    sincospif(2.0f * (float)m / (float)L, &s, &c);
    tw[m] = make_float2(c, S * s);
  }
}

// exp(s 2 pi i q2 k1 / n) for k1 in [0, N1): exact integer angle.
template <int N1, int S>
__device__ __forceinline__ void make_step_twiddles(float2 *st, int q2, int n) {
  for (int k1 = threadIdx.x; k1 < N1; k1 += blockDim.x) {
    const int m = (q2 * k1) & (n - 1);
    float s, c;
    sincospif(2.0f * (float)m / (float)n, &s, &c);
    st[k1] = make_float2(c, S * s);
  }
}

// ----------------------------------------------------------------------
// invert step A: in place on the grid, one CTA per (column tile, q2, plane-pol).
template <int N1>
__global__ void __launch_bounds__(kThreads) k_col_a_inv(const ColGeom cg, float2 *__restrict__ grid) {
  __shared__ float2 buf[N1 * kTC];
  __shared__ float2 tw[N1], st[N1];
  const int p0 = cg.ox + blockIdx.x * kTC;
  const int q2 = blockIdx.y;
  float2 *plane = grid + (int64_t)blockIdx.z * cg.plane;
  make_twiddles<N1, 1>(tw);
  make_step_twiddles<N1, 1>(st, q2, cg.n);
  const int pend = cg.ox + cg.nx;
  for (int e = threadIdx.x; e < N1 * kTC; e += kThreads) {
    const int c = e % kTC, q1 = e / kTC;
    const int p = p0 + c;
    buf[e] = p < pend ? plane[(int64_t)(cg.N2 * q1 + q2) * cg.ngx + p] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  tile_fft<N1, 1>(buf, tw);
  for (int e = threadIdx.x; e < N1 * kTC; e += kThreads) {
    const int c = e % kTC, k1 = e / kTC;
    const int p = p0 + c;
    if (p < pend) plane[(int64_t)(cg.N2 * k1 + q2) * cg.ngx + p] = cmul(buf[e], st[k1]);
  }
}

// invert step B + w-screen + accumulate: one CTA per (column tile, k1); it
// loops over the batch's planes (and pols), accumulating the image pixels it
// owns in registers, and updates acc once.
template <int N2, int NP>
__global__ void __launch_bounds__(kThreads)
    k_col_b_inv(const ColGeom cg, const Geom g, const float2 *__restrict__ grid, int b0, int nb,
                const double *__restrict__ tprime, float *__restrict__ acc, int first) {
  constexpr int EPT = (N2 * kTC + kThreads - 1) / kThreads;
  __shared__ float2 buf[N2 * kTC];
  __shared__ float2 tw[N2];
  const int p0 = cg.ox + blockIdx.x * kTC;
  const int k1 = blockIdx.y;
  const int pend = cg.ox + cg.nx;
  make_twiddles<N2, 1>(tw);
  const int64_t npix = (int64_t)cg.nx * cg.ny;
  int pix[EPT];  // image pixel of element e, or -1
  float a[NP][EPT];
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    const int e = threadIdx.x + i * kThreads;
    pix[i] = -1;
    if (e < N2 * kTC) {
      const int c = e % kTC, k2 = e / kTC;
      const int iy = k1 + cg.N1 * k2 - cg.oy, ix = p0 + c - cg.ox;
      if (iy >= 0 && iy < cg.ny && ix < cg.nx) pix[i] = iy * cg.nx + ix;
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) a[p][i] = (first || pix[i] < 0) ? 0.f : acc[p * npix + pix[i]];
  }
  for (int j = 0; j < nb; ++j) {
    float sn[EPT], cs[EPT];
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      sn[i] = 0.f;
      cs[i] = 1.f;
      if (g.do_w && pix[i] >= 0)
        sincos_2pi((float)plane_turns(g, b0 + j, tprime[pix[i]]), &sn[i], &cs[i]);
    }
#pragma unroll
    for (int pol = 0; pol < NP; ++pol) {
      const float2 *plane = grid + ((int64_t)j * NP + pol) * cg.plane;
      for (int e = threadIdx.x; e < N2 * kTC; e += kThreads) {
        const int c = e % kTC, q2 = e / kTC;
        const int p = p0 + c;
        buf[e] = p < pend ? plane[(int64_t)(cg.N2 * k1 + q2) * cg.ngx + p] : make_float2(0.f, 0.f);
      }
      __syncthreads();
      tile_fft<N2, 1>(buf, tw);
#pragma unroll
      for (int i = 0; i < EPT; ++i) {
        const int e = threadIdx.x + i * kThreads;
        if (pix[i] >= 0) {
          const float2 v = buf[e];
          a[pol][i] += v.x * cs[i] + v.y * sn[i];  // Re(v exp(-i theta))
        }
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < EPT; ++i)
    if (pix[i] >= 0)
#pragma unroll
      for (int p = 0; p < NP; ++p) acc[p * npix + pix[i]] = a[p][i];
}

// predict step A from the corrected image: one CTA per (column tile, q2, pol),
// looping over the batch's planes, so the image tile is read once.
template <int N1, int NP>
__global__ void __launch_bounds__(kThreads)
    k_col_a_pred(const ColGeom cg, const Geom g, const float *__restrict__ img,
                 const double *__restrict__ tprime, int b0, int nb, float2 *__restrict__ grid) {
  constexpr int EPT = (N1 * kTC + kThreads - 1) / kThreads;
  __shared__ float2 buf[N1 * kTC];
  __shared__ float2 tw[N1], st[N1];
  const int p0 = cg.ox + blockIdx.x * kTC;
  const int q2 = blockIdx.y;
  const int pol = blockIdx.z;
  const int pend = cg.ox + cg.nx;
  make_twiddles<N1, -1>(tw);
  make_step_twiddles<N1, -1>(st, q2, cg.n);
  const int64_t npix = (int64_t)cg.nx * cg.ny;
  float v[EPT];
  int pix[EPT];
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    const int e = threadIdx.x + i * kThreads;
    v[i] = 0.f;
    pix[i] = -1;
    if (e < N1 * kTC) {
      const int c = e % kTC, q1 = e / kTC;
      const int iy = cg.N2 * q1 + q2 - cg.oy, ix = p0 + c - cg.ox;
      if (iy >= 0 && iy < cg.ny && ix < cg.nx) {
        pix[i] = iy * cg.nx + ix;
        v[i] = img[pol * npix + pix[i]];
      }
    }
  }
  for (int j = 0; j < nb; ++j) {
    float2 *plane = grid + ((int64_t)j * NP + pol) * cg.plane;
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const int e = threadIdx.x + i * kThreads;
      if (e < N1 * kTC) {
        float sn = 0.f, cs = 1.f;
        if (g.do_w && pix[i] >= 0)
          sincos_2pi((float)plane_turns(g, b0 + j, tprime[pix[i]]), &sn, &cs);
        buf[e] = make_float2(v[i] * cs, v[i] * sn);
      }
    }
    __syncthreads();
    tile_fft<N1, -1>(buf, tw);
    for (int e = threadIdx.x; e < N1 * kTC; e += kThreads) {
      const int c = e % kTC, k1 = e / kTC;
      const int p = p0 + c;
      if (p < pend) plane[(int64_t)(cg.N2 * k1 + q2) * cg.ngx + p] = cmul(buf[e], st[k1]);
    }
    __syncthreads();
  }
}

// predict step B: in place, one CTA per (column tile, k1, plane-pol).
template <int N2>
__global__ void __launch_bounds__(kThreads) k_col_b_pred(const ColGeom cg, float2 *__restrict__ grid) {
  __shared__ float2 buf[N2 * kTC];
  __shared__ float2 tw[N2];
  const int p0 = cg.ox + blockIdx.x * kTC;
  const int k1 = blockIdx.y;
  const int pend = cg.ox + cg.nx;
  float2 *plane = grid + (int64_t)blockIdx.z * cg.plane;
  make_twiddles<N2, -1>(tw);
  for (int e = threadIdx.x; e < N2 * kTC; e += kThreads) {
    const int c = e % kTC, q2 = e / kTC;
    const int p = p0 + c;
    buf[e] = p < pend ? plane[(int64_t)(cg.N2 * k1 + q2) * cg.ngx + p] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  tile_fft<N2, -1>(buf, tw);
  for (int e = threadIdx.x; e < N2 * kTC; e += kThreads) {
    const int c = e % kTC, k2 = e / kTC;
    const int p = p0 + c;
    if (p < pend) plane[(int64_t)(cg.N2 * k1 + k2) * cg.ngx + p] = buf[e];
  }
}

// ----------------------------------------------------------------------
// host side

static int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

bool column_split(int n, int &N1, int &N2) {
  if (n < 256 || n > 32768 || (n & (n - 1))) return false;
  const int lg = ilog2(n);
  const int l1 = lg / 2;  // N1 <= N2
  N1 = 1 << l1;
  N2 = 1 << (lg - l1);
  return N1 >= 16 && N1 <= 128 && N2 <= 256;
}

ColGeom col_geom(const Geom &g) {
  ColGeom cg;
  cg.n = g.ngy;
  column_split(g.ngy, cg.N1, cg.N2);
  cg.ox = (g.ngx - g.nx) / 2;
  cg.oy = (g.ngy - g.ny) / 2;
  cg.nx = g.nx;
  cg.ny = g.ny;
  cg.plane = (int64_t)g.ngx * g.ngy;
  cg.ngx = g.ngx;
  return cg;
}

RowPerm row_perm(const gb_plan *p) {
  RowPerm rp;
  rp.s1 = -1;
  rp.s2 = 0;
  if (p->col_fft) {
    const ColGeom cg = col_geom(p->g);
    rp.s1 = ilog2(cg.N1);
    rp.s2 = ilog2(cg.N2);
  }
  return rp;
}

template <int NP>
static int cols_invert_np(gb_plan *p, float2 *grid, int b0, int nb, float *acc, int first,
                          cudaStream_t s) {
  const Geom &g = p->g;
  const ColGeom cg = col_geom(g);
  const unsigned tiles = (unsigned)((g.nx + kTC - 1) / kTC);
  const double *tprime = p->at<double>(p->off_tprime);
  const double cols = (double)nb * NP * cg.n * g.nx * sizeof(float2);  // central columns
  const double npix = (double)g.nx * g.ny;
  {
    ProfScope ps(kProfColInvA, s, 2.0 * cols);
    const dim3 grd(tiles, cg.N2, nb * NP);
#define GB_COLA(N) k_col_a_inv<N><<<grd, kThreads, 0, s>>>(cg, grid)
    switch (cg.N1) {
      case 16: GB_COLA(16); break;
      case 32: GB_COLA(32); break;
      case 64: GB_COLA(64); break;
      default: GB_COLA(128); break;
    }
#undef GB_COLA
    GB_LAUNCH_CHECK("k_col_a_inv");
  }
  {
    ProfScope ps(kProfColInvB, s,
                 cols + (first ? 1.0 : 2.0) * sizeof(float) * NP * npix + (g.do_w ? 8.0 * npix : 0.0));
    const dim3 grd(tiles, cg.N1);
#define GB_COLB(N) \
  k_col_b_inv<N, NP><<<grd, kThreads, 0, s>>>(cg, g, grid, b0, nb, tprime, acc, first)
    switch (cg.N2) {
      case 16: GB_COLB(16); break;
      case 32: GB_COLB(32); break;
      case 64: GB_COLB(64); break;
      case 128: GB_COLB(128); break;
      default: GB_COLB(256); break;
    }
#undef GB_COLB
    GB_LAUNCH_CHECK("k_col_b_inv");
  }
  return GB_OK;
}

template <int NP>
static int cols_predict_np(gb_plan *p, const float *img, int b0, int nb, float2 *grid,
                           cudaStream_t s) {
  const Geom &g = p->g;
  const ColGeom cg = col_geom(g);
  const unsigned tiles = (unsigned)((g.nx + kTC - 1) / kTC);
  const double *tprime = p->at<double>(p->off_tprime);
  const double cols = (double)nb * NP * cg.n * g.nx * sizeof(float2);
  const double npix = (double)g.nx * g.ny;
  {
    ProfScope ps(kProfColPredA, s, cols + sizeof(float) * NP * npix + (g.do_w ? 8.0 * npix : 0.0));
    const dim3 grd(tiles, cg.N2, NP);
#define GB_COLA(N) k_col_a_pred<N, NP><<<grd, kThreads, 0, s>>>(cg, g, img, tprime, b0, nb, grid)
    switch (cg.N1) {
      case 16: GB_COLA(16); break;
      case 32: GB_COLA(32); break;
      case 64: GB_COLA(64); break;
      default: GB_COLA(128); break;
    }
#undef GB_COLA
    GB_LAUNCH_CHECK("k_col_a_pred");
  }
  {
    ProfScope ps(kProfColPredB, s, 2.0 * cols);
    const dim3 grd(tiles, cg.N1, nb * NP);
#define GB_COLB(N) k_col_b_pred<N><<<grd, kThreads, 0, s>>>(cg, grid)
    switch (cg.N2) {
      case 16: GB_COLB(16); break;
      case 32: GB_COLB(32); break;
      case 64: GB_COLB(64); break;
      case 128: GB_COLB(128); break;
      default: GB_COLB(256); break;
    }
#undef GB_COLB
    GB_LAUNCH_CHECK("k_col_b_pred");
  }
  {
    // zero the columns outside the image: [0, ox) and [ox + nx, ngx) of every row
    const size_t rows = (size_t)nb * NP * g.ngy, pitch = sizeof(float2) * g.ngx;
    const size_t left = sizeof(float2) * cg.ox, right = sizeof(float2) * (g.ngx - cg.ox - g.nx);
    ProfScope ps(kProfZeroMargins, s, (double)rows * (left + right));
    if (left) GB_CUDA(cudaMemset2DAsync(grid, pitch, 0, left, rows, s));
    if (right) GB_CUDA(cudaMemset2DAsync(grid + cg.ox + g.nx, pitch, 0, right, rows, s));
  }
  return GB_OK;
}

int run_cols_invert(gb_plan *p, void *grid, int b0, int nb, float *acc, int first,
                    cudaStream_t s) {
  switch (p->g.NP) {
    case 1: return cols_invert_np<1>(p, (float2 *)grid, b0, nb, acc, first, s);
    case 2: return cols_invert_np<2>(p, (float2 *)grid, b0, nb, acc, first, s);
    default: return cols_invert_np<4>(p, (float2 *)grid, b0, nb, acc, first, s);
  }
}

int run_cols_predict(gb_plan *p, const float *img, int b0, int nb, void *grid, cudaStream_t s) {
  switch (p->g.NP) {
    case 1: return cols_predict_np<1>(p, img, b0, nb, (float2 *)grid, s);
    case 2: return cols_predict_np<2>(p, img, b0, nb, (float2 *)grid, s);
    default: return cols_predict_np<4>(p, img, b0, nb, (float2 *)grid, s);
  }
}

}  // namespace gb
