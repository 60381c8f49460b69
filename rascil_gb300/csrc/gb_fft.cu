// Fused, pruned column transforms of the FP32 form.
//
// A w-plane's 2-D transform is done as row transforms (batched 1-D cuFFT
// over contiguous rows) plus column transforms written here.  Column mode
// applies when the grid height is a power of two and exactly twice the
// image height (sigma = 2), so the image occupies the middle half of every
// column (checkerboarded grids) and only the image's nx columns need
// transforms.  The column length n = N1 N2 is split four-step
// (q = N2 q1 + q2, k = k1 + N1 k2):
//
//   step A  for each q2: the N1-point DFT over q1 of x[N2 q1 + q2], times
//           exp(s 2 pi i q2 k1 / n), stored back at rows N2 k1 + q2;
//   step B  for each k1: the N2-point DFT over the contiguous rows
//           N2 k1 + q2 gives X[k1 + N1 k2].
//
// Each CTA transforms a tile of kCW = 32 adjacent columns (256-byte row
// segments; lane = column).  A column of length N is split N = T M over
// the T warps: warp t holds elements t + T m (m < M) in registers, does an
// M-point DFT in registers, multiplies by exp(s 2 pi i t k1 / N), and one
// exchange through shared memory gives each warp the T-point DFTs of
// outputs k1 + M k2 -- one shared-memory round trip per tile instead of a
// pass per radix stage.
//
// Fusions:
//   invert  (rows first, then columns)  step B never writes the plane back:
//           it keeps only the image rows (outputs k2 in [T/4, 3T/4) of every
//           warp), applies each plane's w-screen and accumulates the image
//           in registers over the batch's planes and pols, with the next
//           tile's loads in flight (cp.async, double-buffered);
//   predict (columns first, then rows)  step A builds its input from the
//           corrected image (inputs m in [M/4, 3M/4) of every warp, zero
//           elsewhere) times each plane's w-screen, and step B writes in
//           place, so physical row N2 k1 + k2 holds logical row k1 + N1 k2;
//           the degridder reads rows through that permutation (RowPerm).
//
// The w-screen of plane k at a pixel is exp(s 2 pi i (A + k D)) with A, D the
// pixel's FP64 phase terms stored as 64-bit fixed-point turns, so the
// per-plane phase is exact integer arithmetic (no FP64 work per plane) and
// only the final sincos of the reduced phase is FP32.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cufft.h>

#include <mutex>

#include "gb_async.cuh"
#include "gb_fft.cuh"

namespace gb {

constexpr int kCW = 32;  // columns per tile: one lane per column

template <int N>
struct ColShape {
  static constexpr int T = N <= 32 ? 4 : (N <= 128 ? 8 : 16);  // warps per column tile
  static constexpr int M = N / T;                              // elements per thread
  static constexpr int THREADS = kCW * T;
  static_assert(M % T == 0 && M % 4 == 0 && T % 4 == 0, "column split");
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float c, float s) {
  return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// a * (s i)
template <int S> __device__ __forceinline__ float2 mul_si(float2 a) {
  return S > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// In-register L-point DFTs in natural order, z_q = sum_p a_p exp(s 2 pi i p q / L).
template <int S> __device__ __forceinline__ void dft4(float2 *a) {
  const float2 s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
  const float2 s13 = cadd(a[1], a[3]), d13 = mul_si<S>(csub(a[1], a[3]));
  a[0] = cadd(s02, s13);
  a[2] = csub(s02, s13);
  a[1] = cadd(d02, d13);
  a[3] = csub(d02, d13);
}

constexpr float kR2 = 0.70710678118654752f;  // cos(pi/4)
constexpr float kC8 = 0.92387953251128674f;  // cos(pi/8)
constexpr float kS8 = 0.38268343236508977f;  // sin(pi/8)

template <int S> __device__ __forceinline__ void dft8(float2 *a) {
  float2 e[4] = {a[0], a[2], a[4], a[6]};
  float2 o[4] = {a[1], a[3], a[5], a[7]};
  dft4<S>(e);
  dft4<S>(o);
  const float2 t0 = o[0], t1 = cmulc(o[1], kR2, S * kR2), t2 = mul_si<S>(o[2]),
               t3 = cmulc(o[3], -kR2, S * kR2);
  a[0] = cadd(e[0], t0);
  a[4] = csub(e[0], t0);
  a[1] = cadd(e[1], t1);
  a[5] = csub(e[1], t1);
  a[2] = cadd(e[2], t2);
  a[6] = csub(e[2], t2);
  a[3] = cadd(e[3], t3);
  a[7] = csub(e[3], t3);
}

// 16 = 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2.
template <int S> __device__ __forceinline__ void dft16(float2 *a) {
  float2 y[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    float2 b[4] = {a[n2], a[4 + n2], a[8 + n2], a[12 + n2]};
    dft4<S>(b);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) y[n2][k1] = b[k1];
  }
  // twiddles exp(s 2 pi i n2 k1 / 16)
  y[1][1] = cmulc(y[1][1], kC8, S * kS8);
  y[1][2] = cmulc(y[1][2], kR2, S * kR2);
  y[1][3] = cmulc(y[1][3], kS8, S * kC8);
  y[2][1] = cmulc(y[2][1], kR2, S * kR2);
  y[2][2] = mul_si<S>(y[2][2]);
  y[2][3] = cmulc(y[2][3], -kR2, S * kR2);
  y[3][1] = cmulc(y[3][1], kS8, S * kC8);
  y[3][2] = cmulc(y[3][2], -kR2, S * kR2);
  y[3][3] = cmulc(y[3][3], -kC8, -S * kS8);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 b[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
    dft4<S>(b);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) a[k1 + 4 * k2] = b[k2];
  }
}

// cos / sin(2 pi k / 32), k < 16
__device__ __constant__ float kCos32[16] = {1.0f, 0.98078528040323043f, 0.92387953251128674f, 0.83146961230254524f, 0.70710678118654757f, 0.55557023301960229f, 0.38268343236508984f, 0.19509032201612833f, 0.0f, -0.19509032201612819f, -0.38268343236508973f, -0.55557023301960196f, -0.70710678118654746f, -0.83146961230254535f, -0.92387953251128674f, -0.98078528040323043f};
__device__ __constant__ float kSin32[16] = {0.0f, 0.19509032201612825f, 0.38268343236508978f, 0.55557023301960218f, 0.70710678118654746f, 0.83146961230254524f, 0.92387953251128674f, 0.98078528040323043f, 1.0f, 0.98078528040323043f, 0.92387953251128674f, 0.83146961230254546f, 0.70710678118654757f, 0.55557023301960218f, 0.38268343236508989f, 0.19509032201612861f};

// 32 = 2 x 16: X[k] = E[k] + w^k O[k], X[k + 16] = E[k] - w^k O[k].
template <int S> __device__ __forceinline__ void dft32(float2 *a) {
  float2 e[16], o[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    e[i] = a[2 * i];
    o[i] = a[2 * i + 1];
  }
  dft16<S>(e);
  dft16<S>(o);
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const float2 t = k == 0 ? o[0] : cmulc(o[k], kCos32[k], S * kSin32[k]);
    a[k] = cadd(e[k], t);
    a[k + 16] = csub(e[k], t);
  }
}

template <int L, int S> __device__ __forceinline__ void dft(float2 *a) {
  if constexpr (L == 4) dft4<S>(a);
  else if constexpr (L == 8) dft8<S>(a);
  else if constexpr (L == 16) dft16<S>(a);
  else dft32<S>(a);
}

// N-point DFT of every column of a tile.  On entry x[m] holds column
// element t + T m of this thread's column (lane c, warp t); on exit
// y[ii][k2] holds output k1 + M k2 with k1 = t + T ii.  xb: N * kCW
// exchange slots; this thread writes only slots (r T + t) kCW + c, r < M,
// before the barrier.  The caller synchronises before xb is reused.
// tw[m] = exp(s 2 pi i m / N).
template <int N, int S>
__device__ __forceinline__ void col_dft(float2 (&x)[ColShape<N>::M], float2 *__restrict__ xb,
                                        const float2 *__restrict__ tw, int t, int c,
                                        float2 (&y)[ColShape<N>::M / ColShape<N>::T]
                                                   [ColShape<N>::T]) {
  constexpr int T = ColShape<N>::T, M = ColShape<N>::M;
  dft<M, S>(x);
#pragma unroll
  for (int k1 = 1; k1 < M; ++k1) x[k1] = cmul(x[k1], tw[t * k1]);
#pragma unroll
  for (int k1 = 0; k1 < M; ++k1) xb[(k1 * T + t) * kCW + c] = x[k1];
  __syncthreads();
#pragma unroll
  for (int ii = 0; ii < M / T; ++ii) {
    const int k1 = t + T * ii;
#pragma unroll
    for (int tt = 0; tt < T; ++tt) y[ii][tt] = xb[(k1 * T + tt) * kCW + c];
    dft<T, S>(y[ii]);
  }
}

// exp(s 2 pi i m / N), m < N, from the n-point table exp(+2 pi i m / n).
template <int N, int S>
__device__ __forceinline__ void load_twiddles(float2 *tw, const float2 *__restrict__ twn, int n) {
  const int step = n / N;
  for (int m = threadIdx.x; m < N; m += blockDim.x) {
    const float2 w = twn[m * step];
    tw[m] = S > 0 ? w : conjf2(w);
  }
}

// sin / cos of plane k's w-screen phase 2 pi (A + k D) at a pixel.
__device__ __forceinline__ void screen_sincos(ulonglong2 ad, int k, float *sn, float *cs) {
  const unsigned long long ph = ad.x + (unsigned long long)(unsigned)k * ad.y;
  const int hi = (int)(unsigned)(ph >> 32);  // turns * 2^32 in [-2^31, 2^31)
  sincospif((float)hi * 0x1p-31f, sn, cs);
}

// The screens of planes b0, b0 + 1, ... at one pixel by rotation: (cs, sn)
// of plane b0 from its exact fixed-point phase, then one complex multiply
// by exp(2 pi i D) per plane (an error of a few FP32 roundings per plane
// step; the batches hold a handful of planes), instead of a sincos per plane.
struct ScreenRot {
  float cs, sn, dc, ds;
  __device__ __forceinline__ void start(ulonglong2 ad, int k) {
    screen_sincos(ad, k, &sn, &cs);
    screen_sincos(make_ulonglong2(ad.y, 0ull), 0, &ds, &dc);
  }
  __device__ __forceinline__ void unit() {
    cs = 1.f;
    sn = 0.f;
    dc = 1.f;
    ds = 0.f;
  }
  __device__ __forceinline__ void next() {
    const float c = cs * dc - sn * ds, s = sn * dc + cs * ds;
    cs = c;
    sn = s;
  }
};

// ----------------------------------------------------------------------
// invert step A: in place, one CTA per (column tile, q2, plane-pol).
template <int N1>
__global__ void __launch_bounds__(ColShape<N1>::THREADS, 3)
    k_cols_a_inv(const ColGeom cg, const float2 *__restrict__ twn, float2 *__restrict__ grid) {
  using CS = ColShape<N1>;
  constexpr int T = CS::T, M = CS::M;
  extern __shared__ float2 smem[];
  float2 *xb = smem, *tw = smem + N1 * kCW;
  const int c = threadIdx.x % kCW, t = threadIdx.x / kCW;
  const int p = cg.ox + blockIdx.x * kCW + c;
  const bool ok = p < cg.ox + cg.nx;
  const int q2 = blockIdx.y;
  float2 *plane = grid + (int64_t)blockIdx.z * cg.plane;
  load_twiddles<N1, 1>(tw, twn, cg.n);
  float2 x[M];
#pragma unroll
  for (int m = 0; m < M; ++m) {
    // rows outside the occupancy mask were never zeroed (nor gridded): load
    // unconditionally (mask and data loads overlap) and select zero
    const int row = cg.N2 * (t + T * m) + q2;
    const float2 v = ok ? plane[(int64_t)row * cg.ngx + p] : make_float2(0.f, 0.f);
    x[m] = cg.row_used(blockIdx.z, row) ? v : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2 y[M / T][T];
  col_dft<N1, 1>(x, xb, tw, t, c, y);
  if (ok) {
#pragma unroll
    for (int ii = 0; ii < M / T; ++ii)
#pragma unroll
      for (int k2 = 0; k2 < T; ++k2) {
        const int o = t + T * ii + M * k2;
        plane[(int64_t)(cg.N2 * o + q2) * cg.ngx + p] = cmul(y[ii][k2], twn[q2 * o]);
      }
  }
}

// invert step B + w-screen + accumulate: one CTA per (column tile, k1).
// The batch's nb x NP plane-pols stream through two shared-memory tile
// buffers filled by TMA (one 2-D box of N2 rows x 32 columns per tile,
// completion on an mbarrier), so the next tile is in flight while this one
// is transformed; the kept outputs accumulate in per-thread shared-memory
// slots.  A wait that runs past its iteration limit records kErrTmaTimeout
// in *status, drains the other buffer (bounded) and returns.
template <int N2, int NP>
__global__ void __launch_bounds__(ColShape<N2>::THREADS, N2 >= 256 ? 1 : 2)
    k_cols_b_inv(const __grid_constant__ CUtensorMap tmap, const ColGeom cg,
                 const float2 *__restrict__ twn, const ulonglong2 *__restrict__ screen, int do_w,
                 int b0, int nb, float *__restrict__ acc, int first,
                 uint32_t *__restrict__ status) {
  using CS = ColShape<N2>;
  constexpr int T = CS::T, M = CS::M, MT = M / T, KL = T / 4, KK = T / 2;
  constexpr int NK = MT * KK;  // kept outputs per thread
  constexpr unsigned kTileBytes = N2 * kCW * sizeof(float2);
  // dynamic shared memory only (TMA destinations at 128-byte offsets):
  // two tiles | twiddles | accumulators | 2 mbarriers | abort flag
  extern __shared__ __align__(128) float2 smem[];
  auto buf = [&](int s) { return smem + (s & 1) * (N2 * kCW); };
  float2 *tw = smem + 2 * N2 * kCW;
  float *sacc = reinterpret_cast<float *>(tw + N2);  // [NP][NK][T][kCW]
  uint64_t *bar = reinterpret_cast<uint64_t *>(sacc + NP * NK * T * kCW);
  int &s_abort = *reinterpret_cast<int *>(bar + 2);
  const int c = threadIdx.x % kCW, t = threadIdx.x / kCW;
  const int p0 = cg.ox + blockIdx.x * kCW;
  const int p = p0 + c;
  const bool ok = p < cg.ox + cg.nx;
  const int ix = p - cg.ox;
  const int k1o = blockIdx.y;
  const int64_t npix = (int64_t)cg.nx * cg.ny;
  const int iters = nb * NP;
  // tile s = plane-pol s of the batch buffer: rows s ngy + N2 k1o + [0, N2)
  auto issue = [&](int s) {
    fence_proxy_async();  // earlier generic writes to the buffer before the async copy
    mbar_expect_tx(&bar[s & 1], kTileBytes);
    tma_load_2d(buf(s), &tmap, p0, s * cg.n + cg.N2 * k1o, &bar[s & 1]);
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    s_abort = 0;
    fence_mbarrier_init();
  }
  load_twiddles<N2, 1>(tw, twn, cg.n);
  __syncthreads();
  if (threadIdx.x == 0) issue(0);
  // kept output e = ii KK + kk: o = t + T ii + M (KL + kk), image row k1o + N1 o - oy
  auto pixel = [&](int e) {
    const int ii = e / KK, kk = e - ii * KK;
    const int o = t + T * ii + M * (KL + kk);
    return (int64_t)(k1o + cg.N1 * o - cg.oy) * cg.nx + ix;
  };
  auto slot = [&](int pol, int e) { return ((pol * NK + e) * T + t) * kCW + c; };
#pragma unroll 1
  for (int pol = 0; pol < NP; ++pol)
#pragma unroll
    for (int e = 0; e < NK; ++e)
      sacc[slot(pol, e)] = (first || !ok) ? 0.f : acc[pol * npix + pixel(e)];
  int s = 0;
  ScreenRot scr[NK];
#pragma unroll
  for (int e = 0; e < NK; ++e) {
    if (do_w && ok)
      scr[e].start(screen[pixel(e)], b0);
    else
      scr[e].unit();
  }
  for (int j = 0; j < nb; ++j) {
    if (j > 0) {
#pragma unroll
      for (int e = 0; e < NK; ++e) scr[e].next();
    }
#pragma unroll 1
    for (int pol = 0; pol < NP; ++pol, ++s) {
      if (threadIdx.x == 0 && s + 1 < iters) issue(s + 1);
      float2 *cur = buf(s);
      if (!mbar_wait(&bar[s & 1], (s >> 1) & 1)) s_abort = 1;
      float2 x[M];
#pragma unroll
      for (int m = 0; m < M; ++m) x[m] = cur[(m * T + t) * kCW + c];
      float2 y[MT][T];
      col_dft<N2, 1>(x, cur, tw, t, c, y);
#pragma unroll
      for (int e = 0; e < NK; ++e) {
        const float2 v = y[e / KK][KL + e % KK];
        sacc[slot(pol, e)] += v.x * scr[e].cs + v.y * scr[e].sn;  // Re(v exp(-i theta))
      }
      __syncthreads();  // tile s consumed before its buffer is refilled
      if (s_abort) {
        if (threadIdx.x == 0) {
          atomicOr(status, kErrTmaTimeout);
          if (s + 1 < iters) mbar_wait(&bar[(s + 1) & 1], ((s + 1) >> 1) & 1);
        }
        return;
      }
    }
  }
  if (ok) {
#pragma unroll 1
    for (int pol = 0; pol < NP; ++pol)
#pragma unroll
      for (int e = 0; e < NK; ++e) acc[pol * npix + pixel(e)] = sacc[slot(pol, e)];
  }
}

// predict step A from the corrected image: one CTA per (column tile, q2);
// loops over the batch's planes and the pols.  The image values (inputs
// m in [M/4, 3M/4) of each thread) and each plane's screens sit in
// per-thread shared-memory slots; the screens of the batch's later planes
// come from the first by rotation (ScreenRot).
template <int N1, int NP>
__global__ void __launch_bounds__(ColShape<N1>::THREADS, 2)
    k_cols_a_pred(const ColGeom cg, const float2 *__restrict__ twn, const float *__restrict__ img,
                  const ulonglong2 *__restrict__ screen, int do_w, int b0, int nb,
                  float2 *__restrict__ grid) {
  using CS = ColShape<N1>;
  constexpr int T = CS::T, M = CS::M, ML = M / 4, MK = M / 2;
  extern __shared__ float2 smem[];
  float2 *xb = smem, *tw = smem + N1 * kCW;
  float2 *st = tw + N1;                                  // exp(-2 pi i q2 o / n), o < N1
  float2 *scr = st + N1;                                 // [MK][T][kCW] (cos, sin)
  float2 *rot = scr + MK * T * kCW;                      // [MK][T][kCW] exp(2 pi i D)
  float *sv = reinterpret_cast<float *>(rot + MK * T * kCW);  // [NP][MK][T][kCW]
  const int c = threadIdx.x % kCW, t = threadIdx.x / kCW;
  const int p = cg.ox + blockIdx.x * kCW + c;
  const bool ok = p < cg.ox + cg.nx;
  const int ix = p - cg.ox;
  const int q2 = blockIdx.y;
  const int64_t npix = (int64_t)cg.nx * cg.ny;
  load_twiddles<N1, -1>(tw, twn, cg.n);
  for (int o = threadIdx.x; o < N1; o += blockDim.x) st[o] = conjf2(twn[q2 * o]);
  // image input mm: row N2 (t + T (ML + mm)) + q2 of the grid, minus oy
  auto pixel = [&](int mm) {
    const int q = cg.N2 * (t + T * (ML + mm)) + q2;
    return (int64_t)(q - cg.oy) * cg.nx + ix;
  };
  auto slot = [&](int mm) { return (mm * T + t) * kCW + c; };
#pragma unroll 1
  for (int pol = 0; pol < NP; ++pol)
#pragma unroll
    for (int mm = 0; mm < MK; ++mm)
      sv[pol * MK * T * kCW + slot(mm)] = ok ? img[pol * npix + pixel(mm)] : 0.f;
  __syncthreads();  // twiddles
  for (int j = 0; j < nb; ++j) {
#pragma unroll
    for (int mm = 0; mm < MK; ++mm) {
      // plane b0 from the fixed-point phase, later planes by rotation
      ScreenRot r;
      if (!(do_w && ok)) {
        r.unit();
      } else if (j == 0) {
        r.start(screen[pixel(mm)], b0);
        rot[slot(mm)] = make_float2(r.dc, r.ds);
      } else {
        const float2 e = scr[slot(mm)], d = rot[slot(mm)];
        r.cs = e.x;
        r.sn = e.y;
        r.dc = d.x;
        r.ds = d.y;
        r.next();
      }
      scr[slot(mm)] = make_float2(r.cs, r.sn);
    }
#pragma unroll 1
    for (int pol = 0; pol < NP; ++pol) {
      float2 x[M];
#pragma unroll
      for (int m = 0; m < M; ++m) x[m] = make_float2(0.f, 0.f);
#pragma unroll
      for (int mm = 0; mm < MK; ++mm) {
        const float2 e = scr[slot(mm)];
        const float v = sv[pol * MK * T * kCW + slot(mm)];
        x[ML + mm] = make_float2(v * e.x, v * e.y);
      }
      float2 y[M / T][T];
      col_dft<N1, -1>(x, xb, tw, t, c, y);
      if (ok) {
        float2 *plane = grid + ((int64_t)j * NP + pol) * cg.plane;
#pragma unroll
        for (int ii = 0; ii < M / T; ++ii)
#pragma unroll
          for (int k2 = 0; k2 < T; ++k2) {
            const int o = t + T * ii + M * k2;
            plane[(int64_t)(cg.N2 * o + q2) * cg.ngx + p] = cmul(y[ii][k2], st[o]);
          }
      }
      __syncthreads();  // exchange slots free again
    }
  }
}

// predict step B: in place, one CTA per (column tile, k1, plane-pol).
template <int N2>
__global__ void __launch_bounds__(ColShape<N2>::THREADS, N2 >= 256 ? 1 : 3)
    k_cols_b_pred(const ColGeom cg, const float2 *__restrict__ twn, float2 *__restrict__ grid) {
  using CS = ColShape<N2>;
  constexpr int T = CS::T, M = CS::M;
  extern __shared__ float2 smem[];
  float2 *xb = smem, *tw = smem + N2 * kCW;
  const int c = threadIdx.x % kCW, t = threadIdx.x / kCW;
  const int p = cg.ox + blockIdx.x * kCW + c;
  const bool ok = p < cg.ox + cg.nx;
  const int k1 = blockIdx.y;
  float2 *plane = grid + (int64_t)blockIdx.z * cg.plane;
  load_twiddles<N2, -1>(tw, twn, cg.n);
  float2 x[M];
#pragma unroll
  for (int m = 0; m < M; ++m)
    x[m] = ok ? plane[(int64_t)(cg.N2 * k1 + t + T * m) * cg.ngx + p] : make_float2(0.f, 0.f);
  __syncthreads();
  float2 y[M / T][T];
  col_dft<N2, -1>(x, xb, tw, t, c, y);
  if (ok) {
#pragma unroll
    for (int ii = 0; ii < M / T; ++ii)
#pragma unroll
      for (int k2 = 0; k2 < T; ++k2)
        plane[(int64_t)(cg.N2 * k1 + t + T * ii + M * k2) * cg.ngx + p] = y[ii][k2];
  }
}

// ----------------------------------------------------------------------
// Row transforms (both forms of the pass over contiguous rows), one CTA
// per row with the whole row in shared memory.  N = R1 R2 R3 by two nested
// four-step splits (all in registers, two shared-memory exchanges):
//   pass 1  unit t < R2 R3 holds x[t + R2 R3 m], m < R1: R1-point DFT,
//           times w_N^(t k1);
//   pass 2  unit (k1, s), s < R3, holds the pass-1 outputs k1 of units
//           s + R3 m': R2-point DFT, times w_(R2 R3)^(s k1');
//   pass 3  unit (k1, k1') holds the pass-2 outputs k1' of units (k1, s):
//           R3-point DFT, giving X[k1 + R1 k1' + R1 R2 k2'].
// Input columns outside [in_lo, in_hi) are taken as zero (predict: only the
// image columns hold data) and only outputs in [out_lo, out_hi) are stored
// (invert: only the image columns are needed).  The first N/2 input cells of
// the next row stream into a shared-memory stage by one bulk copy (mbarrier
// completion) while the current row's passes 2 and 3 and its stores run;
// the rest of the input (invert's second half) is loaded directly, its next
// row prefetched into L2.  A staging wait past its limit records
// kErrTmaTimeout in *status, waits once more (bounded) for the copy in
// flight and returns.  Rows whose (plane, row
// tile) is empty in the occupancy mask are skipped: an invert row there is
// zero (nothing gridded), a predict row there is never degridded.
template <int N> struct RowShape;
template <> struct RowShape<16384> {
  static constexpr int R1 = 32, R2 = 32, R3 = 16, THREADS = 512, MINB = 1;
};
template <> struct RowShape<8192> {
  static constexpr int R1 = 32, R2 = 16, R3 = 16, THREADS = 256, MINB = 2;
};
template <> struct RowShape<4096> {
  static constexpr int R1 = 32, R2 = 16, R3 = 8, THREADS = 128, MINB = 4;
};

struct RowArgs {
  float2 *grid;              // batch buffer: rows of ngx cells
  const uint8_t *mask;       // [nplanes][ntv] occupancy, or null
  const float2 *twx;         // exp(+2 pi i m / ngx), m < ngx
  int64_t nrows;             // nb NP ngy rows in this batch
  int ngy, NP, b0, T, ntv;
  int perm_s1, perm_s2;      // predict rows: logical row of physical r, or -1
  int in_lo, in_hi, out_lo, out_hi;
  uint32_t *status;          // kErrTmaTimeout when a staging wait runs past its limit
};

template <int N, int S>
__global__ void __launch_bounds__(RowShape<N>::THREADS, RowShape<N>::MINB)
    k_rows(const RowArgs ra) {
  using RS = RowShape<N>;
  constexpr int R1 = RS::R1, R2 = RS::R2, R3 = RS::R3, TH = RS::THREADS;
  constexpr int TN = R2 * R3;  // pass-1 units
  constexpr int NA = N / 128;  // two-level twiddle table: w^m = A[m >> 7] B[m & 127]
  static_assert(TN == TH, "one pass-1 unit per thread");
  constexpr int NH = N / 2;  // staged input cells per row
  extern __shared__ __align__(16) float2 smem[];
  float2 *ex = smem;                        // exchange: max(R1 (TN + 1), N) cells
  float2 *ta = smem + R1 * (TN + 1);        // [NA]
  float2 *tb = ta + NA;                     // [128]
  float2 *t2 = tb + 128;                    // [TN]: w_TN^m = w_N^(R1 m)
  float2 *stg = t2 + TN;                    // [NH]: the next row's first input cells
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ int s_abort;
  // staged: input elements m in [m_lo, m_hi) of pass 1 (col = t + TN m), so
  // whole multiples of TN cells (always so for the image-column ranges)
  const int st_lo = ra.in_lo;
  const int st_n = (st_lo % TN == 0 && ra.in_hi % TN == 0) ? min(ra.in_hi - ra.in_lo, NH) : 0;
  const int m_lo = st_lo / TN, m_hi = (st_lo + st_n) / TN;
  const unsigned st_bytes = (unsigned)st_n * (unsigned)sizeof(float2);
  if (threadIdx.x == 0) {
    mbar_init(&s_bar, 1);
    s_abort = 0;
    fence_mbarrier_init();
  }
  for (int i = threadIdx.x; i < NA + 128; i += TH) {
    const float2 w = ra.twx[i < NA ? i * 128 : i - NA];
    (i < NA ? ta[i] : tb[i - NA]) = S > 0 ? w : conjf2(w);
  }
  for (int i = threadIdx.x; i < TN; i += TH) {
    const float2 w = ra.twx[i * R1];
    t2[i] = S > 0 ? w : conjf2(w);
  }
  __syncthreads();
  auto tw = [&](int m) { return cmul(ta[m >> 7], tb[m & 127]); };
  auto used = [&](int64_t row) {
    if (!ra.mask) return true;
    const int sp = (int)(row / ra.ngy), r = (int)(row - (int64_t)sp * ra.ngy);
    const int q = ra.perm_s1 < 0 ? r
                                 : (r >> ra.perm_s2) + ((r & ((1 << ra.perm_s2) - 1)) << ra.perm_s1);
    return ra.mask[(int64_t)(ra.b0 + sp / ra.NP) * ra.ntv + q / ra.T] != 0;
  };
  // the next used row this CTA will transform, prefetched into L2 while
  // this one is transformed (one CTA per SM leaves no other row in flight)
  auto next_used = [&](int64_t row) {
    for (row += gridDim.x; row < ra.nrows && !used(row); row += gridDim.x) {
    }
    return row;
  };
  // the unstaged input of a row, prefetched into L2
  auto prefetch_row = [&](int64_t row) {
    if (threadIdx.x == 0 && row < ra.nrows && st_lo + st_n < ra.in_hi)
      prefetch_l2(ra.grid + row * N + st_lo + st_n,
                  (unsigned)((ra.in_hi - st_lo - st_n) * sizeof(float2)));
  };
  // the staged input of a row (thread 0; the stage's earlier generic reads
  // are ordered before the copy by the barrier and the proxy fence)
  auto stage_row = [&](int64_t row) {
    fence_proxy_async();
    mbar_expect_tx(&s_bar, st_bytes);
    bulk_load(stg, ra.grid + row * N + st_lo, st_bytes, &s_bar);
  };
  const int t = threadIdx.x;
  int64_t row = blockIdx.x;
  if (row < ra.nrows && !used(row)) row = next_used(row);
  __syncthreads();  // the barrier's initialisation before any wait on it
  if (threadIdx.x == 0 && row < ra.nrows && st_n) stage_row(row);
  prefetch_row(row);
  unsigned phase = 0;
  for (; row < ra.nrows;) {
    const int64_t next = next_used(row);
    prefetch_row(next);
    float2 *rp = ra.grid + row * N;
    if (st_n) {
      if (!mbar_wait(&s_bar, phase)) s_abort = 1;
      phase ^= 1u;
    }
    // pass 1
    float2 x[R1];
#pragma unroll
    for (int m = 0; m < R1; ++m) {
      const int col = t + TN * m;
      x[m] = (m >= m_lo && m < m_hi)
                 ? stg[t + TN * (m - m_lo)]
                 : ((col >= ra.in_lo && col < ra.in_hi) ? rp[col] : make_float2(0.f, 0.f));
    }
    dft<R1, S>(x);
    {
      // w^(t k1), k1 < 32, as w^(t (k1 & 7)) w^(8 t (k1 >> 3)): powers of w^t
      // by multiplication (at most 7 roundings) times three table values
      float2 pw[8], qw[4];
      pw[0] = make_float2(1.f, 0.f);
      pw[1] = tw(t);
#pragma unroll
      for (int j = 2; j < 8; ++j) pw[j] = cmul(pw[j - 1], pw[1]);
      qw[0] = pw[0];
#pragma unroll
      for (int i = 1; i < R1 / 8; ++i) qw[i] = tw((8 * t * i) & (N - 1));
      static_assert(R1 == 32, "pass-1 twiddle split");
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) {
        float2 v = x[k1];
        if (k1 & 7) v = cmul(v, pw[k1 & 7]);
        if (k1 >> 3) v = cmul(v, qw[k1 >> 3]);
        ex[k1 * (TN + 1) + t] = v;
      }
    }
    __syncthreads();  // pass-1 exchange written; the stage read by every thread
    if (s_abort) {
      if (threadIdx.x == 0) {
        atomicOr(ra.status, kErrTmaTimeout);
        mbar_wait(&s_bar, phase ^ 1u);  // (bounded) the copy still in flight
      }
      return;
    }
    if (threadIdx.x == 0 && next < ra.nrows && st_n) stage_row(next);
    // pass 2: units u = k1 + R1 s
    constexpr int U2 = R1 * R3 / TH;
    float2 y[U2][R2];
#pragma unroll
    for (int i = 0; i < U2; ++i) {
      const int u = t + TH * i, k1 = u % R1, s = u / R1;
#pragma unroll
      for (int m = 0; m < R2; ++m) y[i][m] = ex[k1 * (TN + 1) + s + R3 * m];
      dft<R2, S>(y[i]);
#pragma unroll
      for (int k = 1; k < R2; ++k) y[i][k] = cmul(y[i][k], t2[s * k]);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < U2; ++i) {
      const int u = t + TH * i, k1 = u % R1, s = u / R1;
#pragma unroll
      for (int k = 0; k < R2; ++k) ex[(k * R3 + s) * R1 + k1] = y[i][k];
    }
    __syncthreads();
    // pass 3: units u = k1 + R1 k1'
    constexpr int U3 = R1 * R2 / TH;
#pragma unroll
    for (int i = 0; i < U3; ++i) {
      const int u = t + TH * i, k1 = u % R1, kp = u / R1;
      float2 z[R3];
#pragma unroll
      for (int s = 0; s < R3; ++s) z[s] = ex[(kp * R3 + s) * R1 + k1];
      dft<R3, S>(z);
#pragma unroll
      for (int k2 = 0; k2 < R3; ++k2) {
        const int o = k1 + R1 * kp + R1 * R2 * k2;
        if (o >= ra.out_lo && o < ra.out_hi) rp[o] = z[k2];
      }
    }
    __syncthreads();  // exchange slots free for the next row
    row = next;
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
  cg.mask = nullptr;
  cg.b0 = 0;
  cg.NP = g.NP;
  cg.T = g.T;
  cg.ntv = g.ntv;
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

// exchange slots + twiddles
template <int N> constexpr size_t smem_one() { return sizeof(float2) * ((size_t)N * kCW + N); }
// + screen slots and image slots (N/2 inputs per column)
template <int N, int NP> constexpr size_t smem_a_pred() {
  return smem_one<N>() + sizeof(float2) * N +
         (2 * sizeof(float2) + sizeof(float) * NP) * (size_t)(N / 2) * kCW;
}
// two tile buffers + twiddles + accumulator slots (N/2 kept outputs per column)
template <int N, int NP> constexpr size_t smem_b_inv() {
  return sizeof(float2) * ((size_t)2 * N * kCW + N) + sizeof(float) * NP * (size_t)(N / 2) * kCW +
         2 * sizeof(uint64_t) + 16;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// link against the driver library).
static PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

// 2-D map over the batch buffer viewed as rows of ngx 8-byte cells
// (B NP ngy rows); box = 32 cells x box_rows rows.
static int make_tile_map(CUtensorMap *map, const gb_plan *p, const float2 *grid, int box_rows) {
  const Geom &g = p->g;
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_tiled();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return GB_ERR_CUDA;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)g.ngx, (cuuint64_t)g.B * g.NP * (cuuint64_t)g.ngy};
  const cuuint64_t strides[1] = {(cuuint64_t)g.ngx * sizeof(float2)};
  const cuuint32_t box[2] = {(cuuint32_t)kCW, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<float2 *>(grid), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) for a %d x %lld grid batch", (int)r, g.ngx,
              (long long)dims[1]);
    return GB_ERR_CUDA;
  }
  return GB_OK;
}

// Kernels whose shared memory exceeds the 48 KB default need the opt-in.
template <int NP>
static int setup_np() {
#define GB_ATTR(K, B) \
  GB_CUDA(cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(B)))
  GB_ATTR((k_cols_b_inv<16, NP>), (smem_b_inv<16, NP>()));
  GB_ATTR((k_cols_b_inv<32, NP>), (smem_b_inv<32, NP>()));
  GB_ATTR((k_cols_b_inv<64, NP>), (smem_b_inv<64, NP>()));
  GB_ATTR((k_cols_b_inv<128, NP>), (smem_b_inv<128, NP>()));
  GB_ATTR((k_cols_b_inv<256, NP>), (smem_b_inv<256, NP>()));
  GB_ATTR(k_cols_b_pred<256>, smem_one<256>());
  GB_ATTR((k_cols_a_pred<16, NP>), (smem_a_pred<16, NP>()));
  GB_ATTR((k_cols_a_pred<32, NP>), (smem_a_pred<32, NP>()));
  GB_ATTR((k_cols_a_pred<64, NP>), (smem_a_pred<64, NP>()));
  GB_ATTR((k_cols_a_pred<128, NP>), (smem_a_pred<128, NP>()));
#undef GB_ATTR
  return GB_OK;
}

int setup_col_kernels(gb_plan *p) {
  if (!p->col_fft) return GB_OK;
  switch (p->g.NP) {
    case 1: return setup_np<1>();
    case 2: return setup_np<2>();
    default: return setup_np<4>();
  }
}

template <int NP>
static int cols_invert_np(gb_plan *p, float2 *grid, int b0, int nb, float *acc, int first,
                          cudaStream_t s) {
  const Geom &g = p->g;
  ColGeom cg = col_geom(g);
  cg.mask = p->at<uint8_t>(p->off_rowmask);
  cg.b0 = b0;
  const unsigned tiles = (unsigned)((g.nx + kCW - 1) / kCW);
  const float2 *twn = p->at<float2>(p->off_twn);
  const ulonglong2 *screen = g.do_w ? p->at<ulonglong2>(p->off_screen) : nullptr;
  const double cols = (double)nb * NP * cg.n * g.nx * sizeof(float2);  // image columns
  const double npix = (double)g.nx * g.ny;
  {
    ProfScope ps(kProfColInvA, s, 2.0 * cols);
    const dim3 grd(tiles, cg.N2, nb * NP);
#define GB_COLA(N)                                                                  \
  k_cols_a_inv<N><<<grd, ColShape<N>::THREADS, smem_one<N>(), s>>>(cg, twn, grid)
    switch (cg.N1) {
      case 16: GB_COLA(16); break;
      case 32: GB_COLA(32); break;
      case 64: GB_COLA(64); break;
      default: GB_COLA(128); break;
    }
#undef GB_COLA
    GB_LAUNCH_CHECK("k_cols_a_inv");
  }
  {
    ProfScope ps(kProfColInvB, s,
                 cols + (first ? 1.0 : 2.0) * sizeof(float) * NP * npix +
                     (g.do_w ? 16.0 * npix : 0.0));
    const dim3 grd(tiles, cg.N1);
    CUtensorMap map;
    int rc = make_tile_map(&map, p, grid, cg.N2);
    if (rc) return rc;
    uint32_t *status = p->status_word();
#define GB_COLB(N)                                                                 \
  k_cols_b_inv<N, NP><<<grd, ColShape<N>::THREADS, smem_b_inv<N, NP>(), s>>>(       \
      map, cg, twn, screen, g.do_w, b0, nb, acc, first, status)
    switch (cg.N2) {
      case 16: GB_COLB(16); break;
      case 32: GB_COLB(32); break;
      case 64: GB_COLB(64); break;
      case 128: GB_COLB(128); break;
      default: GB_COLB(256); break;
    }
#undef GB_COLB
    GB_LAUNCH_CHECK("k_cols_b_inv");
  }
  return GB_OK;
}

template <int NP>
static int cols_predict_np(gb_plan *p, const float *img, int b0, int nb, float2 *grid,
                           cudaStream_t s) {
  const Geom &g = p->g;
  ColGeom cg = col_geom(g);
  cg.mask = p->at<uint8_t>(p->off_rowmask);
  cg.b0 = b0;
  const unsigned tiles = (unsigned)((g.nx + kCW - 1) / kCW);
  const float2 *twn = p->at<float2>(p->off_twn);
  const ulonglong2 *screen = g.do_w ? p->at<ulonglong2>(p->off_screen) : nullptr;
  const double cols = (double)nb * NP * cg.n * g.nx * sizeof(float2);
  const double npix = (double)g.nx * g.ny;
  {
    ProfScope ps(kProfColPredA, s,
                 cols + sizeof(float) * NP * npix + (g.do_w ? 16.0 * npix : 0.0));
    const dim3 grd(tiles, cg.N2);
#define GB_COLA(N)                                                                   \
  k_cols_a_pred<N, NP><<<grd, ColShape<N>::THREADS, smem_a_pred<N, NP>(), s>>>(cg, twn, img, \
                                                                        screen, g.do_w, b0, nb, grid)
    switch (cg.N1) {
      case 16: GB_COLA(16); break;
      case 32: GB_COLA(32); break;
      case 64: GB_COLA(64); break;
      default: GB_COLA(128); break;
    }
#undef GB_COLA
    GB_LAUNCH_CHECK("k_cols_a_pred");
  }
  {
    ProfScope ps(kProfColPredB, s, 2.0 * cols);
    const dim3 grd(tiles, cg.N1, nb * NP);
#define GB_COLB(N) \
  k_cols_b_pred<N><<<grd, ColShape<N>::THREADS, smem_one<N>(), s>>>(cg, twn, grid)
    switch (cg.N2) {
      case 16: GB_COLB(16); break;
      case 32: GB_COLB(32); break;
      case 64: GB_COLB(64); break;
      case 128: GB_COLB(128); break;
      default: GB_COLB(256); break;
    }
#undef GB_COLB
    GB_LAUNCH_CHECK("k_cols_b_pred");
  }
  if (!p->row_fft) {
    // zero the columns outside the image: [0, ox) and [ox + nx, ngx) of every row
    // (k_rows reads only the image columns, so it needs no zeros there)
    const size_t rows = (size_t)nb * NP * g.ngy, pitch = sizeof(float2) * g.ngx;
    const size_t left = sizeof(float2) * cg.ox, right = sizeof(float2) * (g.ngx - cg.ox - g.nx);
    ProfScope ps(kProfZeroMargins, s, (double)rows * (left + right));
    if (left) GB_CUDA(cudaMemset2DAsync(grid, pitch, 0, left, rows, s));
    if (right) GB_CUDA(cudaMemset2DAsync(grid + cg.ox + g.nx, pitch, 0, right, rows, s));
  }
  return GB_OK;
}

// Zero the used rows (mask) of nrows = nb NP ngy rows of ngx cells.
__global__ void k_zero_rows(float2 *__restrict__ grid, const uint8_t *__restrict__ mask,
                            int64_t nrows, int ngx, int ngy, int NP, int b0, int T, int ntv) {
  const int n4 = ngx / 2;  // float4 per row (ngx even)
  for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
    const int sp = (int)(row / ngy), r = (int)(row - (int64_t)sp * ngy);
    if (!mask[(int64_t)(b0 + sp / NP) * ntv + r / T]) continue;
    float4 *dst = reinterpret_cast<float4 *>(grid + row * ngx);
    for (int i = threadIdx.x; i < n4; i += blockDim.x) dst[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

int run_zero_rows(gb_plan *p, void *grid, int b0, int nb, cudaStream_t s) {
  const Geom &g = p->g;
  const int64_t nrows = (int64_t)nb * g.NP * g.ngy;
  const unsigned blocks = (unsigned)std::min<int64_t>(nrows, (int64_t)p->num_sms * 8);
  k_zero_rows<<<blocks, kThreads, 0, s>>>(reinterpret_cast<float2 *>(grid),
                                          p->at<uint8_t>(p->off_rowmask), nrows, g.ngx, g.ngy,
                                          g.NP, b0, g.T, g.ntv);
  GB_LAUNCH_CHECK("k_zero_rows");
  return GB_OK;
}

bool row_kernel_fits(int n) { return n == 4096 || n == 8192 || n == 16384; }

template <int N> constexpr size_t rows_smem() {
  using RS = RowShape<N>;
  return sizeof(float2) *
         ((size_t)RS::R1 * (RS::R2 * RS::R3 + 1) + N / 128 + 128 + RS::R2 * RS::R3 + N / 2);
}

template <int N, int S> static int rows_occupancy(int *per_sm) {
  GB_CUDA(cudaFuncSetAttribute(k_rows<N, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)rows_smem<N>()));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_rows<N, S>,
                                                        RowShape<N>::THREADS, rows_smem<N>()));
  return GB_OK;
}

int setup_row_kernels(gb_plan *p) {
  if (!p->row_fft) return GB_OK;
  int a = 0, b = 0, rc;
  switch (p->g.ngx) {
    case 4096: rc = rows_occupancy<4096, 1>(&a); if (!rc) rc = rows_occupancy<4096, -1>(&b); break;
    case 8192: rc = rows_occupancy<8192, 1>(&a); if (!rc) rc = rows_occupancy<8192, -1>(&b); break;
    default: rc = rows_occupancy<16384, 1>(&a); if (!rc) rc = rows_occupancy<16384, -1>(&b); break;
  }
  if (rc) return rc;
  if (std::min(a, b) < 1) {
    set_error("k_rows cannot launch for rows of %d cells", p->g.ngx);
    return GB_ERR_INVALID_ARG;
  }
  p->row_blocks = std::min(a, b) * p->num_sms;
  return GB_OK;
}

int run_rows(gb_plan *p, void *grid, int b0, int nb, int dir, cudaStream_t s) {
  const Geom &g = p->g;
  const ColGeom cg = col_geom(g);
  RowArgs ra;
  ra.grid = reinterpret_cast<float2 *>(grid);
  ra.mask = p->at<uint8_t>(p->off_rowmask);
  ra.twx = p->at<float2>(p->off_twx);
  ra.nrows = (int64_t)nb * g.NP * g.ngy;
  ra.ngy = g.ngy;
  ra.NP = g.NP;
  ra.b0 = b0;
  ra.T = g.T;
  ra.ntv = g.ntv;
  ra.status = p->status_word();
  if (dir > 0) {  // invert: full rows in, image columns out
    ra.perm_s1 = -1;
    ra.perm_s2 = 0;
    ra.in_lo = 0;
    ra.in_hi = g.ngx;
    ra.out_lo = cg.ox;
    ra.out_hi = cg.ox + g.nx;
  } else {  // predict: image columns in (rest taken as zero), full rows out
    const RowPerm rp = row_perm(p);
    ra.perm_s1 = rp.s1;
    ra.perm_s2 = rp.s2;
    ra.in_lo = cg.ox;
    ra.in_hi = cg.ox + g.nx;
    ra.out_lo = 0;
    ra.out_hi = g.ngx;
  }
  const unsigned blocks = (unsigned)std::min<int64_t>(p->row_blocks, ra.nrows);
#define GB_ROWS(N)                                                                        \
  if (dir > 0)                                                                            \
    k_rows<N, 1><<<blocks, RowShape<N>::THREADS, rows_smem<N>(), s>>>(ra);                \
  else                                                                                    \
    k_rows<N, -1><<<blocks, RowShape<N>::THREADS, rows_smem<N>(), s>>>(ra);
  switch (g.ngx) {
    case 4096: GB_ROWS(4096) break;
    case 8192: GB_ROWS(8192) break;
    default: GB_ROWS(16384) break;
  }
#undef GB_ROWS
  GB_LAUNCH_CHECK("k_rows");
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
