// Invert (ms2dirty): visibilities -> dirty image.
//
// Per call:   k_prep_vis    gather every item's visibilities in bucket order,
//                           apply flags, weights, the pol-frame matrix and the
//                           w-centring rotation; sum the weights per pol.
// Per batch of w-planes:
//             k_grid        one CTA per work chunk (<= 256 items of one
//                           (slab, tile) bucket): the tile's sub-grid lives in
//                           shared memory, each warp spreads one item at a
//                           time over its W x W support (kernel values per
//                           support row/column, exchanged by warp shuffles),
//                           then the sub-grid is flushed to the HBM grid with
//                           vector atomics.  Sparse chunks skip the sub-grid.
//             cuFFT         2-D c2c, e^{+2 pi i}, batched over planes x pols
//             k_screen_acc  reads the central block of each plane, applies the
//                           w-screen exp(-2 pi i w_k (n-1-tc)) and accumulates.
// Once:       k_finalize    multiply by the correction image, write the
//                           requested layout.
#include <cufft.h>

#include "gb_fft.cuh"
#include "gb_plan.cuh"

namespace gb {

template <typename R, int NP>
__global__ void __launch_bounds__(kThreads)
    k_prep_vis(const Geom g, const typename Traits<R>::Item *__restrict__ items,
               const typename Traits<R>::C *__restrict__ vis, int npv,
               const R *__restrict__ wgt, const void *__restrict__ flags, int ftype,
               const PolMat pm, int psf, const double *__restrict__ coords,
               typename Traits<R>::C *__restrict__ cvis, double *__restrict__ sumwt) {
  using C = typename Traits<R>::C;
  double wsum[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) wsum[p] = 0.0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < g.nitems; j += stride) {
    const auto it = items[j];
    const size_t base = (size_t)it.idx * npv;
    // PSF of a phase-shifted plan: unit visibilities carry the w-centring
    // factor alone (the reference rotates before it sets them to one)
    auto ph = it.ph;
    if (coords) {
      R s, c;
      sincos_2pi((R)item_turns(g, coords, coords + 3 * (size_t)g.R, it.idx, false), &s, &c);
      ph.x = c;
      ph.y = -s;
    }
    R m[4];
    for (int q = 0; q < 4; ++q) m[q] = (R)1;
    if (ftype == GB_FLAGS_U8) {
      const uint8_t *f = reinterpret_cast<const uint8_t *>(flags) + base;
      for (int q = 0; q < npv; ++q) m[q] = f[q] ? (R)0 : (R)1;
    } else if (ftype == GB_FLAGS_I64) {
      const int64_t *f = reinterpret_cast<const int64_t *>(flags) + base;
      for (int q = 0; q < npv; ++q) m[q] = f[q] ? (R)0 : (R)1;
    }
    C out[NP];
    if (psf) {
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        out[p].x = p == 0 ? (R)1 : (R)0;
        out[p].y = (R)0;
      }
    } else {
      C v[4];
      for (int q = 0; q < 4; ++q) {
        v[q].x = (R)0;
        v[q].y = (R)0;
      }
      for (int q = 0; q < npv; ++q) {
        const C x = vis[base + q];
        v[q].x = x.x * m[q];
        v[q].y = x.y * m[q];
      }
      if (pm.identity) {
#pragma unroll
        for (int p = 0; p < NP; ++p) out[p] = v[p];
      } else {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          R re = 0, im = 0;
          for (int q = 0; q < npv; ++q) {
            const R mr = pm_re<R>(pm, p * pm.nin + q), mi = pm_im<R>(pm, p * pm.nin + q);
            re += mr * v[q].x - mi * v[q].y;
            im += mr * v[q].y + mi * v[q].x;
          }
          out[p].x = re;
          out[p].y = im;
        }
      }
    }
    // a mirrored item (at -uvw) grids the conjugate value
    const R conj_sign = (it.loc & kLocFlip) ? (R)-1 : (R)1;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const R w = (wgt ? wgt[base + p] : (R)1) * m[p];
      wsum[p] += (double)w;
      const R re = out[p].x * w, im = out[p].y * w * conj_sign;
      C o;
      o.x = re * ph.x - im * ph.y;
      o.y = re * ph.y + im * ph.x;
      cvis[(size_t)j * NP + p] = o;
    }
  }
  if (sumwt) {
    __shared__ double red[kWarps][NP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      double x = wsum[p];
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      if (lane == 0) red[warp][p] = x;
    }
    __syncthreads();
    if (threadIdx.x < NP) {
      double x = 0.0;
      for (int w = 0; w < kWarps; ++w) x += red[w][threadIdx.x];
      atomicAdd(&sumwt[threadIdx.x], x);
    }
  }
}

__device__ __forceinline__ void grid_add(float2 *dst, float re, float im) {
  atomicAdd(dst, make_float2(re, im));
}
__device__ __forceinline__ void grid_add(double2 *dst, double re, double im) {
  atomicAdd(&dst->x, re);
  atomicAdd(&dst->y, im);
}
// Two adjacent cells (dst 16-byte aligned): one vector atomic in FP32.
__device__ __forceinline__ void grid_add2(float2 *dst, float re0, float im0, float re1,
                                          float im1) {
  atomicAdd(reinterpret_cast<float4 *>(dst), make_float4(re0, im0, re1, im1));
}
__device__ __forceinline__ void grid_add2(double2 *dst, double re0, double im0, double re1,
                                          double im1) {
  grid_add(dst, re0, im0);
  grid_add(dst + 1, re1, im1);
}

// Slab range [s_lo, s_hi] whose items reach planes [b0, b0 + nb).
__device__ __forceinline__ void batch_slabs(const Geom &g, int b0, int nb, int &s_lo,
                                            int &s_hi) {
  const int lo = b0 - (g.S + g.W - 2);
  s_lo = lo <= 0 ? 0 : (lo + g.S - 1) / g.S;
  s_hi = min(g.nslabs - 1, (b0 + nb - 1) / g.S);
}

// Fixed-point accumulation for the shared-memory sub-grid: integer shared
// atomics are native, floating-point ones are not.  Each chunk gets its own
// scale (2^30 or 2^61 over the chunk's sum of |value|), so the integer sums
// can neither overflow nor lose more than one part in 2^30 of that bound.
template <typename R> struct FixedAcc;
template <> struct FixedAcc<float> {
  using T = int;
  using T2 = int2;
  static constexpr double kOne = 1073741824.0;  // 2^30
};
template <> struct FixedAcc<double> {
  using T = long long;
  using T2 = longlong2;
  static constexpr double kOne = 2305843009213693952.0;  // 2^61
};
__device__ __forceinline__ int to_fixed(float v) { return __float2int_rn(v); }
__device__ __forceinline__ long long to_fixed(double v) { return __double2ll_rn(v); }
__device__ __forceinline__ void fixed_add(int *p, int v) { atomicAdd(p, v); }
__device__ __forceinline__ void fixed_add(long long *p, long long v) {
  atomicAdd(reinterpret_cast<unsigned long long *>(p), static_cast<unsigned long long>(v));
}

// Shared memory of the tile gridder: the fixed-point sub-grid (2 NP planes
// of the plan's tile layout), then, in the FP32 form, the per-chunk cache of
// every item's kernel values {loc, ku[W], kv[W], kw[W]} and scaled values.
template <typename R> struct GridSmem;
template <> struct GridSmem<float> {
  static constexpr bool kCache = true;
};
template <> struct GridSmem<double> {
  static constexpr bool kCache = false;
};

// The FP32 gridder's spread in integer arithmetic.  For sub-grid chunks
// the item cache holds every item's v kernel values in Q31 (round(kv 2^31),
// saturating at kv = 1), and a lane converts its value times its u and w
// kernel values to fixed point once per item and plane (C = round(2 c), c
// the value at the chunk's fixed-point scale).  A support row's update is
// then round(C K / 2^32) = round(kv c): the high word of one 32 x 32 -> 64
// bit multiply-add with 2^31 as addend, on the integer multiply pipe, where
// a float product and a float-to-integer conversion per row would load the
// conversion unit (a quarter-rate pipe) with two instructions per row.  The
// result is within 1 of round(kv c) in the sub-grid's units, closer than an
// FP32 product of the same magnitudes (a 24-bit mantissa at up to 2^30).
__device__ __forceinline__ int q31_mul_round(int c, int k) {
  int hi;
  asm("{\n\t.reg .b64 t;\n\t.reg .b32 lo;\n\t"
      "mad.wide.s32 t, %1, %2, %3;\n\t"
      "mov.b64 {lo, %0}, t;\n\t}"
      : "=r"(hi)
      : "r"(c), "r"(k), "l"(0x80000000LL));
  return hi;
}

__device__ __forceinline__ int kernel_q31(float kv) {
  return __float2int_rn(kv * 2147483648.0f);  // saturates at 2^31 - 1 for kv = 1
}

// NU (1 or 2) items -- chunk-relative jj0 and jj0 + kWarps -- all with their
// w-support on plane k, spread by one warp into the fixed-point sub-grid.
// WC > 0: the support width as a compile-time constant (no per-row
// predicate beyond the lane's own); WC = 0: W at run time.
template <int NP, int AW, int WC, int NU>
__device__ __forceinline__ void spread_q31_step(const LaneMap<NP, AW> &lm, int W, int k,
                                                int kbase, int jj0,
                                                const float *__restrict__ kc,
                                                const float2 *__restrict__ cc, int *acc,
                                                const TileLayout &L) {
  using LM = LaneMap<NP, AW>;
  constexpr int KS = kcache_stride(AW);
  constexpr int WM = WC > 0 ? WC : AW;                  // rows bound, compile time
  constexpr int NR = (WM + LM::RS - 1) / LM::RS;        // support rows per lane (at most)
  constexpr int NK = LM::RS == 1 ? (WM + 3) / 4 * 4 : 1;  // Q31 row values held
  const bool lane_in = lm.a < W;
  const int im_off = NP * L.plane;
  int kq[NU][NK];
  int cre[NU][LM::NPL], cim[NU][LM::NPL];
  int *pa[NU];
  const int *kjs[NU];
#pragma unroll
  for (int u = 0; u < NU; ++u) {
    const int jj = jj0 + u * kWarps;
    const float *kj = kc + jj * KS;
    kjs[u] = reinterpret_cast<const int *>(kj);
    const uint32_t loc = __float_as_uint(kj[0]);
    const int aw = k - (kbase + (int)((loc >> 16) & 0xffu));  // in [0, W) here
    const float f = 2.f * kj[4 + 2 * AW + aw] * kj[4 + lm.a];   // 2 kw(aw) ku(a)
    if constexpr (LM::RS == 1) {
#pragma unroll
      for (int q = 0; q < NK; q += 4) {
        const int4 t = *reinterpret_cast<const int4 *>(kj + 4 + AW + q);
        kq[u][q] = t.x;
        kq[u][q + 1] = t.y;
        kq[u][q + 2] = t.z;
        kq[u][q + 3] = t.w;
      }
    }
#pragma unroll
    for (int i = 0; i < LM::NPL; ++i) {
      const float2 v = cc[jj * NP + lm.pol(i)];
      cre[u][i] = __float2int_rn(v.x * f);
      cim[u][i] = __float2int_rn(v.y * f);
    }
    const int lu = (int)(loc & 0xffu), lv = (int)((loc >> 8) & 0xffu);
    pa[u] = acc + (lv + lm.r0) * L.pitch + lu + lm.a;
  }
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const int b = lm.r0 + r * LM::RS;
    const bool on = (WC > 0 && LM::RS == 1) ? lane_in : (b < W && lane_in);
    if (on) {
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const int kb = LM::RS == 1 ? kq[u][r] : kjs[u][4 + AW + b];
        int *row = pa[u] + r * LM::RS * L.pitch;
#pragma unroll
        for (int i = 0; i < LM::NPL; ++i) {
          int *cell = row + lm.pol(i) * L.plane;
          atomicAdd(cell, q31_mul_round(cre[u][i], kb));
          atomicAdd(cell + im_off, q31_mul_round(cim[u][i], kb));
        }
      }
    }
  }
}

// The items reaching plane k (chunk-relative [jj_lo, jj_hi), all with their
// w-support on k): warp w takes items jj_lo + w + 2 kWarps i and the items
// kWarps after them, two per step (independent chains of atomics), and a
// last odd item alone.
template <int NP, int AW, int WC>
__device__ __forceinline__ void spread_q31(const LaneMap<NP, AW> &lm, int warp, int W, int k,
                                           int kbase, int jj_lo, int jj_hi,
                                           const float *__restrict__ kc,
                                           const float2 *__restrict__ cc, int *acc,
                                           const TileLayout &L) {
  int j0 = jj_lo + warp;
  for (; j0 + kWarps < jj_hi; j0 += 2 * kWarps)
    spread_q31_step<NP, AW, WC, 2>(lm, W, k, kbase, j0, kc, cc, acc, L);
  if (j0 < jj_hi) spread_q31_step<NP, AW, WC, 1>(lm, W, k, kbase, j0, kc, cc, acc, L);
}

// Support widths with a compile-time instance of the spread (the FP32
// form's defaults: W = 7 at sigma 2 and W = 9 at sigma 1.5 for epsilon
// 1e-5); other widths take the run-time instance.  With the default
// 32-cell tile as well, the sub-grid layout is a compile-time constant, so
// a support row's atomics address the sub-grid by immediate offsets.
template <int NP, int AW>
__device__ __forceinline__ void spread_fixed(const LaneMap<NP, AW> &lm, int warp, int W, int T,
                                             int k, int kbase, int jj_lo, int jj_hi,
                                             const float *__restrict__ kc,
                                             const float2 *__restrict__ cc, int *acc,
                                             const TileLayout &L) {
  if (AW == 8 && W == 7 && T == 32) {
    constexpr TileLayout L32 = tile_layout(32, 7, NP);
    spread_q31<NP, AW, AW == 8 ? 7 : 0>(lm, warp, W, k, kbase, jj_lo, jj_hi, kc, cc, acc, L32);
  } else if (AW == 8 && W == 7) {
    spread_q31<NP, AW, AW == 8 ? 7 : 0>(lm, warp, W, k, kbase, jj_lo, jj_hi, kc, cc, acc, L);
  } else if (AW == 16 && W == 9) {
    spread_q31<NP, AW, AW == 16 ? 9 : 0>(lm, warp, W, k, kbase, jj_lo, jj_hi, kc, cc, acc, L);
  } else {
    spread_q31<NP, AW, 0>(lm, warp, W, k, kbase, jj_lo, jj_hi, kc, cc, acc, L);
  }
}

// Grid one work chunk (up to kChunkItems items of one (w-slab, uv tile)
// bucket) into the planes [b0, b0 + nb) of `grid`: spread every item over
// its W x W support in the shared sub-grid, plane by plane, then flush the
// sub-grid to HBM with float2 atomics and leave it zeroed.  `acc` must be all
// zero on entry (it is on exit); kc / cc are the FP32 item cache; s_red,
// s_scale and s_first (kMaxSlab + 1 entries) are block-shared scratch.
// Every thread of the block calls it.
template <typename R, int NP, int AW>
__device__ __forceinline__ void grid_chunk(
    const Geom &g, const typename Traits<R>::Item *__restrict__ items,
    const typename Traits<R>::C *__restrict__ cvis, const Chunk ch, int b0, int nb,
    typename Traits<R>::C *__restrict__ grid, typename FixedAcc<R>::T *acc, R *kc,
    typename Traits<R>::C *cc, R *s_red, R *s_scale, int *s_first) {
  using C = typename Traits<R>::C;
  using A = typename FixedAcc<R>::T;
  using LM = LaneMap<NP, AW>;
  constexpr bool kCache = GridSmem<R>::kCache;
  const int W = g.W, T = g.T;
  const TileLayout L = tile_layout(T, W, NP);
  constexpr int KS = kcache_stride(AW);  // item cache: loc | ku[AW] | kv[AW] | kw[AW]
  const int SW = L.SW, SW2 = SW * SW;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const LM lm(lane);
  const R scale_u = (R)2 / (R)W;
  const R beta = (R)g.beta;
  const int ntiles = g.ntu * g.ntv;
  const size_t plane = (size_t)g.ngx * g.ngy;
  {
    const int slab = (int)(ch.bucket / (uint32_t)ntiles);
    const int tile = (int)(ch.bucket - (uint32_t)slab * ntiles);
    const int tv = tile / g.ntu, tu = tile - tv * g.ntu;
    const int kbase = slab * g.S;
    // a chunk's items run in order of first w-plane (sort_key): its planes
    // span from its first item's first plane to its last item's last
    const int lk_first = (int)((items[ch.begin].loc >> 16) & 0xffu);
    const int lk_last = (int)((items[ch.end - 1].loc >> 16) & 0xffu);
    const int k_lo = max(kbase + lk_first, b0);
    const int k_hi = min(min(kbase + lk_last + W, g.nplanes), b0 + nb);
    if (k_lo >= k_hi) return;  // (block-uniform) no item reaches this batch's planes
    const int n = (int)(ch.end - ch.begin);
    const bool direct = n * W * W < SW2;
    // chunk scale for the fixed-point sub-grid: 2^k / sum_j max |component|,
    // summed in the form's precision (the FP32 form: a sum low by a few
    // parts in 10^7 at most, against the factor-2 headroom of the 2^30
    // bound in int32, so no cell sum can overflow)
    R scale = (R)0, inv = (R)0;
    if (!direct) {
      R m = (R)0;
      for (uint32_t j = ch.begin + threadIdx.x; j < ch.end; j += kThreads) {
        R mj = (R)0;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const C v = cvis[(size_t)j * NP + p];
          mj = fmax(mj, fmax(fabs(v.x), fabs(v.y)));
        }
        m += mj;
      }
      for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
      if (lane == 0) s_red[warp] = m;
      __syncthreads();
      // one thread forms the scale and its inverse
      if (threadIdx.x == 0) {
        R S = (R)0;
        for (int w = 0; w < kWarps; ++w) S += s_red[w];
        constexpr R kOne = (R)FixedAcc<R>::kOne, kInvOne = (R)(1.0 / FixedAcc<R>::kOne);
        s_scale[0] = S > (R)0 ? kOne / S : (R)0;
        s_scale[1] = S > (R)0 ? S * kInvOne : (R)0;
      }
      __syncthreads();
      scale = s_scale[0];
      inv = s_scale[1];
    }
    __syncthreads();  // s_red, s_scale and s_ci are reused by the next chunk
    // A bucket's items run in order of first w-plane inside the slab (lk):
    // s_first[l] = the first item of the chunk with lk >= l, so the items
    // reaching plane k (lk in [k - kbase - W + 1, k - kbase]) are one run.
    for (int jj = threadIdx.x; jj < n; jj += kThreads) {
      const int lk = (int)((items[ch.begin + jj].loc >> 16) & 0xffu);
      const int lkp = jj == 0 ? -1 : (int)((items[ch.begin + jj - 1].loc >> 16) & 0xffu);
      for (int q = lkp + 1; q <= lk; ++q) s_first[q] = jj;
      if (jj == n - 1)
        for (int q = lk + 1; q <= g.S; ++q) s_first[q] = n;
    }
    if constexpr (!kCache) __syncthreads();
    if constexpr (kCache) {
      const R f = direct ? (R)1 : scale;
      for (int jj = threadIdx.x; jj < n; jj += kThreads) {
        const auto it = items[ch.begin + jj];
        R *c = kc + jj * KS;
        c[0] = __uint_as_float(it.loc);
#pragma unroll
        for (int a = 0; a < AW; ++a) {
          const bool in = a < W;
          c[4 + a] = in ? es_kernel(((R)a - it.du) * scale_u, beta) : (R)0;
          // v values: float for direct chunks, Q31 for the sub-grid spread
          const R kv = in ? es_kernel(((R)a - it.dv) * scale_u, beta) : (R)0;
          c[4 + AW + a] = direct ? kv : __int_as_float(kernel_q31(kv));
          c[4 + 2 * AW + a] = in ? (g.do_w ? es_kernel(((R)a - it.dwf) * scale_u, beta) : (R)1)
                                 : (R)0;
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          C v = cvis[(size_t)(ch.begin + jj) * NP + p];
          v.x *= f;
          v.y *= f;
          cc[jj * NP + p] = v;
        }
      }
      __syncthreads();
    }
    for (int k = k_lo; k < k_hi; ++k) {
      C *gplane = grid + (size_t)(k - b0) * NP * plane;
      const int lk_lo = max(0, k - kbase - W + 1), lk_hi = min(g.S - 1, k - kbase);
      const uint32_t j_lo = ch.begin + (uint32_t)s_first[lk_lo];
      const uint32_t j_hi = lk_lo <= lk_hi ? ch.begin + (uint32_t)s_first[lk_hi + 1] : j_lo;
      if constexpr (kCache) {
        if (!direct)
          spread_fixed<NP, AW>(lm, warp, W, T, k, kbase, (int)(j_lo - ch.begin),
                               (int)(j_hi - ch.begin), kc, cc, acc, L);
      }
      for (uint32_t j = j_lo + warp; j < j_hi && (!kCache || direct); j += kWarps) {
        const int jj = (int)(j - ch.begin);
        R fw, ku, kv_lane = (R)0;
        uint32_t loc;
        C c[LM::NPL];
        if constexpr (kCache) {
          const R *kj = kc + jj * KS;
          loc = __float_as_uint(kj[0]);
          const int aw = k - (kbase + (int)((loc >> 16) & 0xffu));
          if (aw < 0 || aw >= W) continue;
          fw = kj[4 + 2 * AW + aw];
          ku = kj[4 + lm.a];  // zero for a >= W
          if (lane >= 16 && lane - 16 < W) kv_lane = kj[4 + AW + lane - 16];
#pragma unroll
          for (int i = 0; i < LM::NPL; ++i) {
            c[i] = cc[jj * NP + lm.pol(i)];
            c[i].x *= fw;
            c[i].y *= fw;
          }
        } else {
          const auto it = items[j];
          loc = it.loc;
          const int aw = k - (kbase + (int)((it.loc >> 16) & 0xffu));
          if (aw < 0 || aw >= W) continue;
          fw = g.do_w ? es_kernel(((R)aw - it.dwf) * scale_u, beta) : (R)1;
          // lanes 0..15 hold the u kernel values, 16..31 the v values
          if (lane < 16) {
            if (lane < W) kv_lane = es_kernel(((R)lane - it.du) * scale_u, beta);
          } else if (lane - 16 < W) {
            kv_lane = es_kernel(((R)(lane - 16) - it.dv) * scale_u, beta);
          }
          ku = __shfl_sync(0xffffffffu, kv_lane, lm.a);
#pragma unroll
          for (int i = 0; i < LM::NPL; ++i) {
            c[i] = cvis[(size_t)j * NP + lm.pol(i)];
            const R f = fw * (direct ? (R)1 : scale);
            c[i].x *= f;
            c[i].y *= f;
          }
        }
        const int lu = (int)(loc & 0xffu), lv = (int)((loc >> 8) & 0xffu);
        // the lane's column kernel value folded into its values once per
        // item and plane: a support row then costs one multiply per part
#pragma unroll
        for (int i = 0; i < LM::NPL; ++i) {
          c[i].x *= ku;
          c[i].y *= ku;
        }
        constexpr int kMaxRows = (AW + LM::RS - 1) / LM::RS;  // W <= AW: unrolled, predicated
        const int cell0 = (lv + lm.r0) * L.pitch + lu + lm.a;
#pragma unroll
        for (int r = 0; r < kMaxRows; ++r) {
          const int b = lm.r0 + r * LM::RS;
          const R kv = __shfl_sync(0xffffffffu, kv_lane, 16 + min(b, W - 1));
          if (b < W && lm.a < W) {
            if (direct) {
              int p = tu * T + lu + lm.a;
              if (p >= g.ngx) p -= g.ngx;
              int q = tv * T + lv + b;
              if (q >= g.ngy) q -= g.ngy;
              const R f = ((p + q) & 1) ? -kv : kv;
#pragma unroll
              for (int i = 0; i < LM::NPL; ++i)
                grid_add(&gplane[lm.pol(i) * plane + (size_t)q * g.ngx + p], f * c[i].x,
                         f * c[i].y);
            } else {
              const int cell = cell0 + r * LM::RS * L.pitch;
#pragma unroll
              for (int i = 0; i < LM::NPL; ++i) {
                const int pl = lm.pol(i);
                fixed_add(&acc[pl * L.plane + cell], to_fixed(kv * c[i].x));
                fixed_add(&acc[(NP + pl) * L.plane + cell], to_fixed(kv * c[i].y));
              }
            }
          }
        }
      }
      if (!direct) {
        __syncthreads();
        // flush: fixed point -> float, add to HBM, and leave the sub-grid
        // zeroed.  A thread takes two adjacent cells (x even): one 16-byte
        // vector atomic per pol for both (tile origins, x and the grid width
        // are even, so p is even and the pair never straddles the wrap).  For
        // odd SW the last pair's second cell is row padding, never written,
        // so it adds zero.
        const int hp = (SW + 1) >> 1;  // cell pairs per sub-grid row
        for (int i = threadIdx.x; i < SW * hp; i += kThreads) {
          const int y = i / hp, x = 2 * (i - y * hp);
          const int cell = y * L.pitch + x;
          int p = tu * T + x;
          while (p >= g.ngx) p -= g.ngx;
          int q = tv * T + y;
          while (q >= g.ngy) q -= g.ngy;
          const R sgn = ((p + q) & 1) ? -inv : inv;  // the pair's second cell: -sgn
#pragma unroll
          for (int pol = 0; pol < NP; ++pol) {
            // the pair as one 8-byte (FP32 form) or 16-byte (FP64 form)
            // shared access: cell is even, and so are the pitch and the
            // plane stride
            using A2 = typename FixedAcc<R>::T2;
            A2 *are = reinterpret_cast<A2 *>(acc + pol * L.plane + cell);
            A2 *aim = reinterpret_cast<A2 *>(acc + (NP + pol) * L.plane + cell);
            const A2 re = *are, im = *aim;
            if ((re.x | re.y | im.x | im.y) != 0) {
              *are = A2{0, 0};
              *aim = A2{0, 0};
              grid_add2(&gplane[pol * plane + (size_t)q * g.ngx + p], sgn * (R)re.x,
                        sgn * (R)im.x, -sgn * (R)re.y, -sgn * (R)im.y);
            }
          }
        }
        __syncthreads();
      }
    }
  }
}

template <typename R, int NP, int AW>
__global__ void __launch_bounds__(kThreads)
    k_grid(const Geom g, const typename Traits<R>::Item *__restrict__ items,
           const typename Traits<R>::C *__restrict__ cvis, const Chunk *__restrict__ chunks,
           const uint32_t *__restrict__ chunk_off, int b0, int nb,
           typename Traits<R>::C *__restrict__ grid, uint32_t *__restrict__ counter) {
  using C = typename Traits<R>::C;
  using A = typename FixedAcc<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  A *acc = reinterpret_cast<A *>(smem_raw);  // [re pols | im pols][SW][pitch]
  const TileLayout L = tile_layout(g.T, g.W, NP);
  R *kc = reinterpret_cast<R *>(acc + 2 * NP * L.plane);  // [kChunkItems][kcache_stride]
  C *cc = reinterpret_cast<C *>(kc + kChunkItems * kcache_stride(AW));  // [kChunkItems][NP]
  const int ntiles = g.ntu * g.ntv;
  int s_lo, s_hi;
  batch_slabs(g, b0, nb, s_lo, s_hi);
  const uint32_t c_begin = chunk_off[(int64_t)s_lo * ntiles];
  const uint32_t c_end = chunk_off[(int64_t)(s_hi + 1) * ntiles];
  for (int i = threadIdx.x; i < 2 * NP * L.plane; i += kThreads) acc[i] = 0;
  __shared__ uint32_t s_ci;
  __shared__ R s_red[kWarps];
  __shared__ R s_scale[2];
  __shared__ int s_first[kMaxSlab + 1];
  for (;;) {
    if (threadIdx.x == 0) s_ci = c_begin + atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t ci = s_ci;
    if (ci >= c_end) break;
    grid_chunk<R, NP, AW>(g, items, cvis, chunks[ci], b0, nb, grid, acc, kc, cc, s_red, s_scale,
                          s_first);
  }
}

template <typename R, int NP>
__global__ void __launch_bounds__(kThreads)
    k_screen_acc(const Geom g, const typename Traits<R>::C *__restrict__ grid, int b0, int nb,
                 const double *__restrict__ tprime, R *__restrict__ acc, int first) {
  using C = typename Traits<R>::C;
  const int64_t npix = (int64_t)g.nx * g.ny;
  const int ox = (g.ngx - g.nx) / 2, oy = (g.ngy - g.ny) / 2;
  const size_t plane = (size_t)g.ngx * g.ngy;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix; i += stride) {
    const int iy = (int)(i / g.nx), ix = (int)(i - (int64_t)iy * g.nx);
    R a[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) a[p] = first ? (R)0 : acc[p * npix + i];
    const size_t gi = (size_t)(iy + oy) * g.ngx + (ix + ox);
    if (g.do_w) {
      PlaneTurns pt;
      pt.start(g, b0, tprime[i]);
      for (int j = 0; j < nb; ++j) {
        R s, c;
        sincos_2pi(pt.turns(j, (R)0), &s, &c);
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const C v = grid[((size_t)j * NP + p) * plane + gi];
          a[p] += v.x * c + v.y * s;
        }
      }
    } else {
#pragma unroll
      for (int p = 0; p < NP; ++p) a[p] += grid[(size_t)p * plane + gi].x;
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[p * npix + i] = a[p];
  }
}

// out = acc * corr in the requested layout (32 x 32 tiles, transposed
// through shared memory for ducc0's [x][y] order).
template <typename R>
__global__ void k_finalize(const Geom g, const R *__restrict__ acc, const R *__restrict__ corr,
                           R *__restrict__ out, int layout) {
  __shared__ R tile[32][33];
  const int64_t npix = (int64_t)g.nx * g.ny;
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32, p = blockIdx.z;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int iy = by + j, ix = bx + threadIdx.x;
    if (iy < g.ny && ix < g.nx) {
      const int64_t i = (int64_t)iy * g.nx + ix;
      const R v = acc[p * npix + i] * corr[i];
      if (layout == GB_LAYOUT_YX)
        out[p * npix + i] = v;
      else
        tile[j][threadIdx.x] = v;
    }
  }
  if (layout == GB_LAYOUT_XY) {
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
      const int ix = bx + j, iy = by + threadIdx.x;
      if (iy < g.ny && ix < g.nx) out[p * npix + (int64_t)ix * g.ny + iy] = tile[threadIdx.x][j];
    }
  }
}

template <typename R> static cufftResult fft_exec(cufftHandle h, void *data, int dir);
template <> cufftResult fft_exec<float>(cufftHandle h, void *data, int dir) {
  return cufftExecC2C(h, (cufftComplex *)data, (cufftComplex *)data, dir);
}
template <> cufftResult fft_exec<double>(cufftHandle h, void *data, int dir) {
  return cufftExecZ2Z(h, (cufftDoubleComplex *)data, (cufftDoubleComplex *)data, dir);
}

static int fft_one(gb_plan *p, cufftHandle h, void *data, int dir, cudaStream_t s,
                   const char *what) {
  if (cufftSetStream(h, s) != CUFFT_SUCCESS) {
    set_error("cufftSetStream failed");
    return GB_ERR_CUFFT;
  }
  const cufftResult r = p->precision == GB_FP64 ? fft_exec<double>(h, data, dir)
                                                : fft_exec<float>(h, data, dir);
  if (r != CUFFT_SUCCESS) {
    const cudaError_t e = cudaGetLastError();
    set_error("cufftExec (%s) failed (cufft status %d, CUDA %s)", what, (int)r,
              cudaGetErrorString(e));
    return GB_ERR_CUFFT;
  }
  return GB_OK;
}

// 2-D transform of nb planes x NP pols (in place).
int run_fft(gb_plan *p, int nb, void *data, int dir, cudaStream_t s) {
  const cufftHandle h = nb == p->g.B ? p->fft_full : p->fft_rem;
  const int rc = fft_one(p, h, data, dir, s, dir == CUFFT_INVERSE ? "inverse" : "forward");
  if (rc) return rc;
  GB_LAUNCH_CHECK("cufftExec");
  return GB_OK;
}

// Shared memory of k_grid / k_degrid: 2 NP planes of 4- or 8-byte words.
size_t tile_smem_bytes(const gb_plan *p) {
  const TileLayout L = tile_layout(p->g.T, p->g.W, p->g.NP);
  return (size_t)2 * p->g.NP * L.plane * real_bytes(p->precision);
}

// k_grid: the sub-grid plus, in the FP32 form, the per-chunk item cache.
size_t grid_smem_bytes(const gb_plan *p) {
  size_t b = tile_smem_bytes(p);
  if (p->precision == GB_FP32)
    b += (size_t)kChunkItems *
         (kcache_stride(group_lanes(p->g.W)) * sizeof(float) + p->g.NP * sizeof(float2));
  return b;
}

// The invert driver in steps (a batch of plans interleaves them across
// plans: gb_batch.cu).  begin: per-item values; per w-plane batch bi: zero,
// grid, transform (+ screen and accumulation); end: correction and layout.
template <typename R, int NP>
static int inv_begin_impl(gb_plan *p, const void *vis, int npv, const void *wgt,
                          const void *flags, int ftype, const PolMat &pm, int psf, double *sumwt,
                          cudaStream_t s) {
  using C = typename Traits<R>::C;
  using Item = typename Traits<R>::Item;
  const Geom &g = p->g;
  char *tmp = p->ws + p->off_temp;
  C *cvis = reinterpret_cast<C *>(tmp + p->c_cvis);
  uint32_t *counters = p->at<uint32_t>(p->off_counters);
  const Item *items = p->at<Item>(p->off_items);
  GB_CUDA(cudaMemsetAsync(counters, 0, 4 * (size_t)p->nbatches, s));
  if (sumwt) GB_CUDA(cudaMemsetAsync(sumwt, 0, sizeof(double) * NP, s));
  const unsigned item_blocks = (unsigned)std::min<int64_t>(
      ((int64_t)g.nitems + kThreads - 1) / kThreads, (int64_t)p->num_sms * 16);
  const double fb = ftype == GB_FLAGS_I64 ? 8.0 : (ftype == GB_FLAGS_U8 ? 1.0 : 0.0);
  const double per = sizeof(Item) + (psf ? 0.0 : npv * sizeof(C)) +
                     (wgt ? NP * sizeof(R) : 0.0) + npv * fb + NP * sizeof(C);
  ProfScope ps(kProfPrepVis, s, per * (double)g.nitems);
  k_prep_vis<R, NP><<<item_blocks, kThreads, 0, s>>>(
      g, items, reinterpret_cast<const C *>(vis), npv, reinterpret_cast<const R *>(wgt), flags,
      ftype, pm, psf, psf && g.shifted ? p->at<const double>(p->off_coords) : nullptr, cvis,
      sumwt);
  GB_LAUNCH_CHECK("k_prep_vis");
  return GB_OK;
}

template <typename R, int NP>
static int inv_zero_impl(gb_plan *p, int bi, cudaStream_t s) {
  using C = typename Traits<R>::C;
  const Geom &g = p->g;
  C *grid = reinterpret_cast<C *>(p->ws + p->off_temp + p->c_grid);
  const int b0 = bi * g.B, nb = std::min(g.B, g.nplanes - b0);
  const double gbytes = (double)sizeof(C) * nb * NP * (double)g.ngx * g.ngy;
  if (p->col_fft) {  // only rows the gridder writes; column step A skips the rest
    ProfScope ps(kProfGridZero, s, p->used_rows(b0, nb) * gbytes);
    return run_zero_rows(p, grid, b0, nb, s);
  }
  ProfScope ps(kProfGridZero, s, gbytes);
  GB_CUDA(cudaMemsetAsync(grid, 0, (size_t)gbytes, s));
  return GB_OK;
}

// Algorithmic bytes and updates of gridding batch bi (profiling).
template <typename R, int NP>
static void grid_counts(const gb_plan *p, int bi, double *bytes, double *updates) {
  using C = typename Traits<R>::C;
  using Item = typename Traits<R>::Item;
  const Geom &g = p->g;
  const int b0 = bi * g.B, nb = std::min(g.B, g.nplanes - b0);
  const double gbytes = (double)sizeof(C) * nb * NP * (double)g.ngx * g.ngy;
  // items and their gridded values read once; every grid cell of the
  // (plane, tile) pairs they reach read and written once (the float2
  // atomic flush is a read-modify-write), else the rows they reach
  const double cells = p->touched_cells(b0, nb);
  const double gmove = cells > 0.0 ? 2.0 * cells * NP * sizeof(C) : p->used_rows(b0, nb) * gbytes;
  *bytes = (double)p->batch_items(b0, nb) * (sizeof(Item) + NP * sizeof(C)) + gmove;
  *updates = p->item_planes(b0, nb) * g.W * g.W * NP;
}

template <typename R, int NP>
static int inv_grid_impl(gb_plan *p, int bi, cudaStream_t s) {
  using C = typename Traits<R>::C;
  using Item = typename Traits<R>::Item;
  const Geom &g = p->g;
  char *tmp = p->ws + p->off_temp;
  C *grid = reinterpret_cast<C *>(tmp + p->c_grid);
  const C *cvis = reinterpret_cast<const C *>(tmp + p->c_cvis);
  uint32_t *counters = p->at<uint32_t>(p->off_counters);
  const Item *items = p->at<Item>(p->off_items);
  const Chunk *chunks = p->at<Chunk>(p->off_chunks);
  const uint32_t *chunk_off = p->at<uint32_t>(p->off_chunk_off);
  const int b0 = bi * g.B, nb = std::min(g.B, g.nplanes - b0);
  const size_t smem = grid_smem_bytes(p);
  double bytes = 0.0, updates = 0.0;
  if (prof_on()) grid_counts<R, NP>(p, bi, &bytes, &updates);
  ProfScope ps(kProfGrid, s, bytes, updates);
  if (group_lanes(g.W) == 8)
    k_grid<R, NP, 8><<<p->grid_blocks, kThreads, smem, s>>>(g, items, cvis, chunks, chunk_off,
                                                            b0, nb, grid, counters + bi);
  else
    k_grid<R, NP, 16><<<p->grid_blocks, kThreads, smem, s>>>(g, items, cvis, chunks, chunk_off,
                                                             b0, nb, grid, counters + bi);
  GB_LAUNCH_CHECK("k_grid");
  return GB_OK;
}

template <typename R, int NP>
static int inv_transform_impl(gb_plan *p, int bi, cudaStream_t s) {
  using C = typename Traits<R>::C;
  const Geom &g = p->g;
  char *tmp = p->ws + p->off_temp;
  C *grid = reinterpret_cast<C *>(tmp + p->c_grid);
  R *acc = reinterpret_cast<R *>(tmp + p->c_img);
  const int b0 = bi * g.B, nb = std::min(g.B, g.nplanes - b0);
  const double gbytes = (double)sizeof(C) * nb * NP * (double)g.ngx * g.ngy;
  const int64_t npix = (int64_t)g.nx * g.ny;
  int rc;
  if (p->row_fft) {
    // used rows: read, image half written
    ProfScope ps(kProfRowsInv, s, 1.5 * p->used_rows(b0, nb) * gbytes);
    rc = run_rows(p, grid, b0, nb, 1, s);
  } else {
    ProfScope ps(kProfFftInv, s, 2.0 * gbytes);
    rc = run_fft(p, nb, grid, CUFFT_INVERSE, s);
  }
  if (rc) return rc;
  if constexpr (std::is_same<R, float>::value) {
    if (p->col_fft)  // rows done; columns + screen + accumulate
      return run_cols_invert(p, grid, b0, nb, acc, bi == 0, s);
  }
  const unsigned pix_blocks = (unsigned)std::min<int64_t>((npix + kThreads - 1) / kThreads,
                                                          (int64_t)p->num_sms * 32);
  ProfScope ps(kProfScreenAcc, s,
               (double)sizeof(C) * nb * NP * npix + (bi ? 2.0 : 1.0) * sizeof(R) * NP * npix);
  k_screen_acc<R, NP><<<pix_blocks, kThreads, 0, s>>>(g, grid, b0, nb,
                                                       p->at<double>(p->off_tprime), acc, bi == 0);
  GB_LAUNCH_CHECK("k_screen_acc");
  return GB_OK;
}

template <typename R, int NP>
static int inv_end_impl(gb_plan *p, void *dirty, int layout, cudaStream_t s) {
  const Geom &g = p->g;
  const R *acc = reinterpret_cast<const R *>(p->ws + p->off_temp + p->c_img);
  const R *corr = p->at<R>(p->off_corr);
  const int64_t npix = (int64_t)g.nx * g.ny;
  dim3 fb((g.nx + 31) / 32, (g.ny + 31) / 32, NP);
  ProfScope ps(kProfFinalize, s, 3.0 * sizeof(R) * NP * (double)npix);
  k_finalize<R><<<fb, dim3(32, 8), 0, s>>>(g, acc, corr, reinterpret_cast<R *>(dirty), layout);
  GB_LAUNCH_CHECK("k_finalize");
  return GB_OK;
}

template <typename R, int NP>
static int ms2dirty_impl(gb_plan *p, const void *vis, int npv, const void *wgt,
                         const void *flags, int ftype, const PolMat &pm, int psf, void *dirty,
                         int layout, double *sumwt, cudaStream_t s) {
  int rc = inv_begin_impl<R, NP>(p, vis, npv, wgt, flags, ftype, pm, psf, sumwt, s);
  for (int bi = 0; !rc && bi < p->nbatches; ++bi) {
    rc = inv_zero_impl<R, NP>(p, bi, s);
    if (!rc) rc = inv_grid_impl<R, NP>(p, bi, s);
    if (!rc) rc = inv_transform_impl<R, NP>(p, bi, s);
  }
  if (!rc) rc = inv_end_impl<R, NP>(p, dirty, layout, s);
  return rc;
}

// Dispatch on (precision, NP) for the step entry points.
#define GB_INV_DISPATCH(p, CALL)                     \
  do {                                               \
    if ((p)->precision == GB_FP64) {                 \
      switch ((p)->g.NP) {                           \
        case 1: { using R = double; constexpr int NP = 1; return CALL; } \
        case 2: { using R = double; constexpr int NP = 2; return CALL; } \
        default: { using R = double; constexpr int NP = 4; return CALL; } \
      }                                              \
    }                                                \
    switch ((p)->g.NP) {                             \
      case 1: { using R = float; constexpr int NP = 1; return CALL; } \
      case 2: { using R = float; constexpr int NP = 2; return CALL; } \
      default: { using R = float; constexpr int NP = 4; return CALL; } \
    }                                                \
  } while (0)

int inv_begin(gb_plan *p, const void *vis, int npv, const void *wgt, const void *flags,
              int ftype, const PolMat &pm, int psf, double *sumwt, cudaStream_t s) {
  GB_INV_DISPATCH(p, (inv_begin_impl<R, NP>(p, vis, npv, wgt, flags, ftype, pm, psf, sumwt, s)));
}
int inv_zero(gb_plan *p, int bi, cudaStream_t s) {
  GB_INV_DISPATCH(p, (inv_zero_impl<R, NP>(p, bi, s)));
}
int inv_transform(gb_plan *p, int bi, cudaStream_t s) {
  GB_INV_DISPATCH(p, (inv_transform_impl<R, NP>(p, bi, s)));
}
int inv_end(gb_plan *p, void *dirty, int layout, cudaStream_t s) {
  GB_INV_DISPATCH(p, (inv_end_impl<R, NP>(p, dirty, layout, s)));
}

// ---------------------------------------------------------------------
// Many plans' gridding in one persistent launch (FP32 form).  The work
// queue is the concatenation of every job's chunk range (the chunks of the
// slabs its batch of w-planes reaches); each CTA takes the next index from
// one atomic counter, finds its job by the prefix of chunk counts (formed by
// every CTA at start from the plans' chunk offsets on the device, so the
// host needs no copy) and grids that chunk into the job's planes.
template <int NP, int AW>
__global__ void __launch_bounds__(kThreads)
    k_grid_jobs(const __grid_constant__ GridJobs jobs, int acc_words, int ks_max,
                uint32_t *__restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int *acc = reinterpret_cast<int *>(smem_raw);
  float *kc = reinterpret_cast<float *>(acc + acc_words);
  float2 *cc = reinterpret_cast<float2 *>(kc + kChunkItems * ks_max);
  __shared__ uint32_t s_wbeg[kMaxJobs + 1], s_cbeg[kMaxJobs];
  __shared__ uint32_t s_w;
  __shared__ int s_j;
  __shared__ float s_red[kWarps];
  __shared__ float s_scale[2];
  __shared__ int s_first[kMaxSlab + 1];
  if (threadIdx.x == 0) {
    uint32_t w = 0;
    for (int j = 0; j < jobs.n; ++j) {
      const GridJob &jb = jobs.job[j];
      const int ntiles = jb.g.ntu * jb.g.ntv;
      int s_lo, s_hi;
      batch_slabs(jb.g, jb.b0, jb.nb, s_lo, s_hi);
      const uint32_t c0 = jb.chunk_off[(int64_t)s_lo * ntiles];
      const uint32_t c1 = jb.chunk_off[(int64_t)(s_hi + 1) * ntiles];
      s_wbeg[j] = w;
      s_cbeg[j] = c0;
      w += c1 > c0 ? c1 - c0 : 0u;
    }
    s_wbeg[jobs.n] = w;
  }
  for (int i = threadIdx.x; i < acc_words; i += kThreads) acc[i] = 0;
  __syncthreads();
  const uint32_t total = s_wbeg[jobs.n];
  for (;;) {
    if (threadIdx.x == 0) {
      const uint32_t w = atomicAdd(counter, 1u);
      int j = 0;
      while (j + 1 < jobs.n && s_wbeg[j + 1] <= w) ++j;
      s_w = w;
      s_j = j;
    }
    __syncthreads();
    const uint32_t w = s_w;
    if (w >= total) break;
    const GridJob &jb = jobs.job[s_j];
    const uint32_t ci = s_cbeg[s_j] + (w - s_wbeg[s_j]);
    grid_chunk<float, NP, AW>(jb.g, reinterpret_cast<const ItemF *>(jb.items),
                              reinterpret_cast<const float2 *>(jb.cvis), jb.chunks[ci], jb.b0,
                              jb.nb, reinterpret_cast<float2 *>(jb.grid), acc, kc, cc, s_red,
                              s_scale, s_first);
  }
}

// Fill one job of a multi-plan gridding launch from a bound FP32 plan.
int grid_job(gb_plan *p, int bi, GridJob &jb) {
  if (p->precision != GB_FP32 || !p->bound || bi < 0 || bi >= p->nbatches) {
    set_error("grid_job: needs a bound FP32 plan and a batch index in range");
    return GB_ERR_INVALID_ARG;
  }
  char *tmp = p->ws + p->off_temp;
  jb.g = p->g;
  jb.items = p->at<ItemF>(p->off_items);
  jb.cvis = tmp + p->c_cvis;
  jb.chunks = p->at<Chunk>(p->off_chunks);
  jb.chunk_off = p->at<uint32_t>(p->off_chunk_off);
  jb.grid = tmp + p->c_grid;
  jb.b0 = bi * p->g.B;
  jb.nb = std::min(p->g.B, p->g.nplanes - jb.b0);
  return GB_OK;
}

// One launch over `jobs` (all of one NP and lane width); `counter` must be
// zero.  Blocks: the occupancy of the largest job's shared memory.
int launch_grid_jobs(const GridJobs &jobs, int num_sms, uint32_t *counter, double bytes,
                     double updates, cudaStream_t s) {
  if (jobs.n < 1 || jobs.n > kMaxJobs) {
    set_error("launch_grid_jobs: %d jobs (1..%d)", jobs.n, kMaxJobs);
    return GB_ERR_INVALID_ARG;
  }
  const int NP = jobs.job[0].g.NP, AW = group_lanes(jobs.job[0].g.W);
  int acc_words = 0, ks_max = 0;
  for (int j = 0; j < jobs.n; ++j) {
    const Geom &g = jobs.job[j].g;
    if (g.NP != NP || group_lanes(g.W) != AW) {
      set_error("launch_grid_jobs: jobs of one launch share NP and lane width");
      return GB_ERR_INVALID_ARG;
    }
    const TileLayout L = tile_layout(g.T, g.W, g.NP);
    acc_words = std::max(acc_words, 2 * NP * L.plane);
    ks_max = std::max(ks_max, kcache_stride(AW));
  }
  const size_t smem = (size_t)acc_words * 4 + (size_t)kChunkItems * (ks_max * 4 + NP * 8);
  ProfScope ps(kProfGrid, s, bytes, updates);
#define GB_GJ(NPV, AWV)                                                                      \
  {                                                                                          \
    auto k = k_grid_jobs<NPV, AWV>;                                                          \
    GB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
    int per_sm = 0;                                                                          \
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem));      \
    if (per_sm < 1) {                                                                        \
      set_error("k_grid_jobs cannot launch with %zu bytes of shared memory", smem);         \
      return GB_ERR_INVALID_ARG;                                                             \
    }                                                                                        \
    k<<<per_sm * num_sms, kThreads, smem, s>>>(jobs, acc_words, ks_max, counter);            \
  }
  if (AW == 8) {
    if (NP == 1) GB_GJ(1, 8) else if (NP == 2) GB_GJ(2, 8) else GB_GJ(4, 8)
  } else {
    if (NP == 1) GB_GJ(1, 16) else if (NP == 2) GB_GJ(2, 16) else GB_GJ(4, 16)
  }
#undef GB_GJ
  GB_LAUNCH_CHECK("k_grid_jobs");
  return GB_OK;
}

// Profiling counts of gridding batch bi of a plan (0 while profiling is off).
void grid_job_counts(const gb_plan *p, int bi, double *bytes, double *updates) {
  *bytes = 0.0;
  *updates = 0.0;
  if (!prof_on()) return;
  switch (p->g.NP) {
    case 1: grid_counts<float, 1>(p, bi, bytes, updates); break;
    case 2: grid_counts<float, 2>(p, bi, bytes, updates); break;
    default: grid_counts<float, 4>(p, bi, bytes, updates); break;
  }
}

int run_ms2dirty(gb_plan *p, const void *vis, int npv, const void *wgt, const void *flags,
                 int ftype, const PolMat &pm, int psf, void *dirty, int layout, double *sumwt,
                 cudaStream_t s) {
#define GB_CASE(R, NP)                                                                   \
  return ms2dirty_impl<R, NP>(p, vis, npv, wgt, flags, ftype, pm, psf, dirty, layout, sumwt, \
                              s)
  if (p->precision == GB_FP64) {
    switch (p->g.NP) {
      case 1: GB_CASE(double, 1);
      case 2: GB_CASE(double, 2);
      default: GB_CASE(double, 4);
    }
  }
  switch (p->g.NP) {
    case 1: GB_CASE(float, 1);
    case 2: GB_CASE(float, 2);
    default: GB_CASE(float, 4);
  }
#undef GB_CASE
}

template <typename R, int NP, int AW>
static int setup_grid_aw(gb_plan *p) {
  const size_t smem = grid_smem_bytes(p);
  GB_CUDA(cudaFuncSetAttribute(k_grid<R, NP, AW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_grid<R, NP, AW>, kThreads,
                                                        smem));
  if (per_sm < 1) {
    set_error("k_grid cannot launch with %zu bytes of shared memory", smem);
    return GB_ERR_INVALID_ARG;
  }
  p->grid_blocks = per_sm * p->num_sms;
  return GB_OK;
}

template <typename R, int NP>
static int setup_grid_impl(gb_plan *p) {
  return group_lanes(p->g.W) == 8 ? setup_grid_aw<R, NP, 8>(p) : setup_grid_aw<R, NP, 16>(p);
}

int setup_grid_kernels(gb_plan *p) {
  if (p->precision == GB_FP64) {
    switch (p->g.NP) {
      case 1: return setup_grid_impl<double, 1>(p);
      case 2: return setup_grid_impl<double, 2>(p);
      default: return setup_grid_impl<double, 4>(p);
    }
  }
  switch (p->g.NP) {
    case 1: return setup_grid_impl<float, 1>(p);
    case 2: return setup_grid_impl<float, 2>(p);
    default: return setup_grid_impl<float, 4>(p);
  }
}

}  // namespace gb
