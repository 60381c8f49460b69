// Predict (dirty2ms): model image -> visibilities.
//
// Per call:   k_prep_image  image * correction, into [pol][y][x] order.
// Per batch of w-planes:
//             k_screen_pad  every grid cell of every plane in the batch is
//                           written once: the central block gets
//                           image * exp(+2 pi i w_k (n-1-tc)), the rest 0
//                           (no separate memset pass).
//             cuFFT         2-D c2c, e^{-2 pi i}
//             k_degrid_warp one CTA per work chunk (FP32 form): every item's
//                           kernel values cached once per chunk; per plane a
//                           warp per item reads its W x W support straight
//                           from the grid (a lane group's eight lanes read
//                           one 64-byte row segment), weights it and sums
//                           the lanes with shuffles into the item's running
//                           sums.  k_degrid (FP64 form) stages each plane's
//                           sub-grid in shared memory instead.  The
//                           epilogue rotates back by exp(+2 pi i w tc),
//                           conjugates mirrored items, applies the pol-frame
//                           matrix and weights and writes (first batch of
//                           the item) or accumulates (later batches) in place.
#include <cufft.h>

#include "gb_async.cuh"
#include "gb_fft.cuh"
#include "gb_plan.cuh"

namespace gb {

int run_fft(gb_plan *p, int nb, void *data, int dir, cudaStream_t s);
size_t tile_smem_bytes(const gb_plan *p);
int setup_grid_kernels(gb_plan *p);

template <typename R>
__global__ void k_prep_image(const Geom g, const R *__restrict__ dirty, int layout,
                             const R *__restrict__ corr, R *__restrict__ img) {
  __shared__ R tile[32][33];
  const int64_t npix = (int64_t)g.nx * g.ny;
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32, p = blockIdx.z;
  if (layout == GB_LAYOUT_XY) {
    // read dirty[p][x][y] rows (y fastest) into the tile
    for (int j = threadIdx.y; j < 32; j += 8) {
      const int ix = bx + j, iy = by + threadIdx.x;
      if (ix < g.nx && iy < g.ny) tile[threadIdx.x][j] = dirty[p * npix + (int64_t)ix * g.ny + iy];
    }
    __syncthreads();
  }
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int iy = by + j, ix = bx + threadIdx.x;
    if (iy < g.ny && ix < g.nx) {
      const int64_t i = (int64_t)iy * g.nx + ix;
      const R v = layout == GB_LAYOUT_XY ? tile[j][threadIdx.x] : dirty[p * npix + i];
      img[p * npix + i] = v * corr[i];
    }
  }
}

template <typename R, int NP>
__global__ void __launch_bounds__(kThreads)
    k_screen_pad(const Geom g, const R *__restrict__ img, const double *__restrict__ tprime,
                 int b0, int nb, typename Traits<R>::C *__restrict__ grid) {
  using C = typename Traits<R>::C;
  const int64_t npix = (int64_t)g.nx * g.ny;
  const int ox = (g.ngx - g.nx) / 2, oy = (g.ngy - g.ny) / 2;
  const int64_t plane = (int64_t)g.ngx * g.ngy;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < plane; i += stride) {
    const int my = (int)(i / g.ngx), mx = (int)(i - (int64_t)my * g.ngx);
    const int ix = mx - ox, iy = my - oy;
    if (ix >= 0 && ix < g.nx && iy >= 0 && iy < g.ny) {
      const int64_t pi = (int64_t)iy * g.nx + ix;
      R v[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) v[p] = img[p * npix + pi];
      if (g.do_w) {
        PlaneTurns pt;
        pt.start(g, b0, tprime[pi]);
        for (int j = 0; j < nb; ++j) {
          R s, c;
          sincos_2pi(pt.turns(j, (R)0), &s, &c);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            C z;
            z.x = v[p] * c;
            z.y = v[p] * s;
            grid[((int64_t)j * NP + p) * plane + i] = z;
          }
        }
      } else {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          C z;
          z.x = v[p];
          z.y = (R)0;
          grid[(int64_t)p * plane + i] = z;
        }
      }
    } else {
      C z;
      z.x = (R)0;
      z.y = (R)0;
      for (int j = 0; j < nb; ++j)
#pragma unroll
        for (int p = 0; p < NP; ++p) grid[((int64_t)j * NP + p) * plane + i] = z;
    }
  }
}

template <typename R>
__device__ __forceinline__ R warp_sum(R x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

template <typename R, int NP, int AW>
__global__ void __launch_bounds__(kThreads)
    k_degrid(const Geom g, const typename Traits<R>::Item *__restrict__ items,
             const Chunk *__restrict__ chunks, const uint32_t *__restrict__ chunk_off, int b0,
             int nb, const typename Traits<R>::C *__restrict__ grid,
             typename Traits<R>::C *__restrict__ vis, int npv, const R *__restrict__ wgt,
             const PolMat pm, const RowPerm rp, uint32_t *__restrict__ counter) {
  using C = typename Traits<R>::C;
  using LM = LaneMap<NP, AW>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R *sg = reinterpret_cast<R *>(smem_raw);  // [re pols | im pols][SW][pitch]
  const int W = g.W, T = g.T;
  const TileLayout L = tile_layout(T, W, NP);
  const int SW = L.SW, SW2 = SW * SW;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const LM lm(lane);
  const R scale_u = (R)2 / (R)W;
  const R beta = (R)g.beta;
  const int ntiles = g.ntu * g.ntv;
  const int64_t plane = (int64_t)g.ngx * g.ngy;
  const int wk = g.do_w ? W : 1;
  const int lo = b0 - (g.S + W - 2);
  const int s_lo = lo <= 0 ? 0 : (lo + g.S - 1) / g.S;
  const int s_hi = min(g.nslabs - 1, (b0 + nb - 1) / g.S);
  const uint32_t c_begin = chunk_off[(int64_t)s_lo * ntiles];
  const uint32_t c_end = chunk_off[(int64_t)(s_hi + 1) * ntiles];
  __shared__ uint32_t s_ci;
  for (;;) {
    if (threadIdx.x == 0) s_ci = c_begin + atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t ci = s_ci;
    __syncthreads();
    if (ci >= c_end) break;
    const Chunk ch = chunks[ci];
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
    const int n = (int)(ch.end - ch.begin);
    const bool direct = n * W * W < SW2;
    R ar[NP], ai[NP];  // lane i: running sums of item warp*32 + i
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      ar[p] = (R)0;
      ai[p] = (R)0;
    }
    for (int k = k_lo; k < k_hi; ++k) {
      const C *gplane = grid + (int64_t)(k - b0) * NP * plane;
      if (!direct) {
        // stage the sub-grid (checkerboard sign applied), split re / im
        for (int i = threadIdx.x; i < SW2; i += kThreads) {
          const int y = i / SW, x = i - y * SW;
          int p = tu * T + x;
          while (p >= g.ngx) p -= g.ngx;
          int q = tv * T + y;
          while (q >= g.ngy) q -= g.ngy;
          const R sgn = ((p + q) & 1) ? (R)-1 : (R)1;
          const int cell = y * L.pitch + x;
          const int64_t row = (int64_t)rp.row(q) * g.ngx;
#pragma unroll
          for (int pol = 0; pol < NP; ++pol) {
            const C v = gplane[pol * plane + row + p];
            sg[pol * L.plane + cell] = sgn * v.x;
            sg[(NP + pol) * L.plane + cell] = sgn * v.y;
          }
        }
        __syncthreads();
      }
      for (int i = 0; i < 32; ++i) {
        const uint32_t j = ch.begin + (uint32_t)(warp * 32 + i);
        if (j >= ch.end) break;
        const auto it = items[j];
        const int aw = k - (kbase + (int)((it.loc >> 16) & 0xffu));
        if (aw < 0 || aw >= wk) continue;
        R kv_lane = (R)0;
        if (lane < 16) {
          if (lane < W) kv_lane = es_kernel(((R)lane - it.du) * scale_u, beta);
        } else if (lane - 16 < W) {
          kv_lane = es_kernel(((R)(lane - 16) - it.dv) * scale_u, beta);
        }
        const R ku = __shfl_sync(0xffffffffu, kv_lane, lm.a);
        const int lu = (int)(it.loc & 0xffu), lv = (int)((it.loc >> 8) & 0xffu);
        R sr[LM::NPL], si[LM::NPL];
#pragma unroll
        for (int q = 0; q < LM::NPL; ++q) {
          sr[q] = (R)0;
          si[q] = (R)0;
        }
        constexpr int kMaxRows = (AW + LM::RS - 1) / LM::RS;  // W <= AW: unrolled, predicated
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
              for (int qq = 0; qq < LM::NPL; ++qq) {
                const C v = gplane[lm.pol(qq) * plane + (int64_t)rp.row(q) * g.ngx + p];
                sr[qq] += f * v.x;
                si[qq] += f * v.y;
              }
            } else {
              const int cell = (lv + b) * L.pitch + lu + lm.a;
#pragma unroll
              for (int qq = 0; qq < LM::NPL; ++qq) {
                sr[qq] += kv * sg[lm.pol(qq) * L.plane + cell];
                si[qq] += kv * sg[(NP + lm.pol(qq)) * L.plane + cell];
              }
            }
          }
        }
        // sum over the support columns (within a group) and, if several
        // groups share a polarisation, over their row subsets
#pragma unroll
        for (int qq = 0; qq < LM::NPL; ++qq) {
          R xr = sr[qq] * ku, xi = si[qq] * ku;
#pragma unroll
          for (int o = 1; o < AW; o <<= 1) {
            xr += __shfl_xor_sync(0xffffffffu, xr, o);
            xi += __shfl_xor_sync(0xffffffffu, xi, o);
          }
          if (NP < LM::G) {
#pragma unroll
            for (int o = AW * NP; o < 32; o <<= 1) {
              xr += __shfl_xor_sync(0xffffffffu, xr, o);
              xi += __shfl_xor_sync(0xffffffffu, xi, o);
            }
          }
          sr[qq] = xr;
          si[qq] = xi;
        }
        const R fw = g.do_w ? es_kernel(((R)aw - it.dwf) * scale_u, beta) : (R)1;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const int holder = (p % LM::G) * AW;
          const int slot = NP >= LM::G ? p / LM::G : 0;
          const R vr = __shfl_sync(0xffffffffu, sr[slot], holder);
          const R vi = __shfl_sync(0xffffffffu, si[slot], holder);
          if (lane == i) {
            ar[p] += fw * vr;
            ai[p] += fw * vi;
          }
        }
      }
      if (!direct) __syncthreads();
    }
    // epilogue: lane owns item warp*32 + lane of the chunk
    const uint32_t j = ch.begin + (uint32_t)(warp * 32 + lane);
    if (j < ch.end) {
      const auto it = items[j];
      const int k0 = kbase + (int)((it.loc >> 16) & 0xffu);
      if (k0 + wk > b0 && k0 < b0 + nb) {
        C v[NP];
        // a mirrored item (at -uvw) predicts the conjugate
        const R conj_sign = (it.loc & kLocFlip) ? (R)-1 : (R)1;
#pragma unroll
        for (int p = 0; p < NP; ++p) {  // multiply by conj(ph) = exp(+2 pi i w tc)
          v[p].x = ar[p] * it.ph.x + ai[p] * it.ph.y;
          v[p].y = (ai[p] * it.ph.x - ar[p] * it.ph.y) * conj_sign;
        }
        const size_t base = (size_t)it.idx * npv;
        const bool first = k0 >= b0;
        for (int q = 0; q < npv; ++q) {
          C o;
          if (pm.identity) {
            o = v[q < NP ? q : NP - 1];
          } else {
            R re = 0, im = 0;
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              const R mr = pm_re<R>(pm, q * pm.nin + p), mi = pm_im<R>(pm, q * pm.nin + p);
              re += mr * v[p].x - mi * v[p].y;
              im += mr * v[p].y + mi * v[p].x;
            }
            o.x = re;
            o.y = im;
          }
          if (wgt) {
            const R w = wgt[base + q];
            o.x *= w;
            o.y *= w;
          }
          if (first) {
            vis[base + q] = o;
          } else {
            C prev = vis[base + q];
            prev.x += o.x;
            prev.y += o.y;
            vis[base + q] = prev;
          }
        }
      }
    }
  }
}

// FP32 degridder, warp per item, reading the grid directly (no staging
// pass).  A CTA takes a work chunk (up to kChunkItems items of one (w-slab,
// uv tile) bucket).  Once per chunk it caches in shared memory every item's
// kernel values -- the u and v values with the checkerboard sign (-1)^(p+q)
// folded in, and the w values -- and the chunk's grid rows (wrapped, in the
// grid's row order, times the row length) and columns.  Then per w-plane k
// each warp takes the items reaching k whose chunk index is congruent to the
// warp modulo the warp count (an item always meets the same warp, so its
// running sums need no barrier between planes), two items at a time: lane
// (g, a) reads column a of the item's support rows of its pols straight
// from the grid -- the eight lanes of a group read eight adjacent cells of
// one row, one 64-byte segment -- weights them by the v values, folds in its
// u value, and the lanes of a group are summed by shuffles.  The tile's
// cells of one plane stay in L1 while the chunk's items pass over them.
// Per item-plane: W reads and 2 W FMAs per lane and one shuffle reduction,
// with no shared-memory staging and no per-plane barrier.  The epilogue
// (thread i, item i) rotates back by exp(+2 pi i w tc), conjugates mirrored
// items, applies the pol-frame matrix and weights and writes (the item's
// first batch) or accumulates (later batches).
template <int NP, int AW>
__device__ __forceinline__ void degrid_warp_chunk(
    const Geom &g, const ItemF *__restrict__ items, const Chunk ch, int b0, int nb,
    const float2 *__restrict__ grid, float2 *__restrict__ vis, int npv,
    const float *__restrict__ wgt, const PolMat &pm, const RowPerm &rp, float *kc, float2 *sacc,
    int *s_first, int *s_rowoff, int *s_col) {
  using LM = LaneMap<NP, AW>;
  constexpr int KS = kcache_stride(AW);
  constexpr int kMaxRows = (AW + LM::RS - 1) / LM::RS;
  const int W = g.W, T = g.T, SW = T + W - 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const LM lm(lane);
  const bool lane_in = lm.a < W;
  const float scale_u = 2.f / (float)W;
  const float beta = (float)g.beta;
  const int ntiles = g.ntu * g.ntv;
  const int64_t plane = (int64_t)g.ngx * g.ngy;
  const int wk = g.do_w ? W : 1;
  const int slab = (int)(ch.bucket / (uint32_t)ntiles);
  const int tile = (int)(ch.bucket - (uint32_t)slab * ntiles);
  const int tv = tile / g.ntu, tu = tile - tv * g.ntu;
  const int kbase = slab * g.S;
  // a chunk's items run in order of first w-plane (sort_key): its planes
  // span from its first item's first plane to its last item's last
  const int lk_first = (int)((items[ch.begin].loc >> 16) & 0xffu);
  const int lk_last = (int)((items[ch.end - 1].loc >> 16) & 0xffu);
  const int k_lo = max(kbase + lk_first, b0);
  const int k_hi = min(min(kbase + lk_last + wk, g.nplanes), b0 + nb);
  if (k_lo >= k_hi) return;  // (block-uniform) no item reaches this batch's planes
  const int n = (int)(ch.end - ch.begin);
  for (int i = threadIdx.x; i < 2 * SW; i += kThreads) {
    if (i < SW) {
      int q = tv * T + i;
      while (q >= g.ngy) q -= g.ngy;
      s_rowoff[i] = rp.row(q) * g.ngx;
    } else {
      int pc = tu * T + (i - SW);
      while (pc >= g.ngx) pc -= g.ngx;
      s_col[i - SW] = pc;
    }
  }
  const int tpar = ((tu + tv) * T) & 1;  // checkerboard parity of the tile origin
  for (int jj = threadIdx.x; jj < n; jj += kThreads) {
    const ItemF it = items[ch.begin + jj];
    float *c = kc + jj * KS;
    c[0] = __uint_as_float(it.loc);
    const int lu = (int)(it.loc & 0xffu), lv = (int)((it.loc >> 8) & 0xffu);
#pragma unroll
    for (int a = 0; a < AW; ++a) {
      const bool in = a < W;
      const float x = in ? es_kernel(((float)a - it.du) * scale_u, beta) : 0.f;
      const float y = in ? es_kernel(((float)a - it.dv) * scale_u, beta) : 0.f;
      c[4 + a] = ((lu + a + tpar) & 1) ? -x : x;
      c[4 + AW + a] = ((lv + a) & 1) ? -y : y;
      c[4 + 2 * AW + a] = in ? (g.do_w ? es_kernel(((float)a - it.dwf) * scale_u, beta) : 1.f)
                             : 0.f;
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) sacc[jj * NP + p] = make_float2(0.f, 0.f);
    // s_first[l] = the first item with lk >= l (the items reaching plane k
    // are then one run)
    const int lk = (int)((it.loc >> 16) & 0xffu);
    const int lkp = jj == 0 ? -1 : (int)((items[ch.begin + jj - 1].loc >> 16) & 0xffu);
    for (int q = lkp + 1; q <= lk; ++q) s_first[q] = jj;
    if (jj == n - 1)
      for (int q = lk + 1; q <= g.S; ++q) s_first[q] = n;
  }
  __syncthreads();
  for (int k = k_lo; k < k_hi; ++k) {
    const float2 *gplane = grid + (int64_t)(k - b0) * NP * plane;
    const int lk_lo = max(0, k - kbase - wk + 1), lk_hi = min(g.S - 1, k - kbase);
    if (lk_lo > lk_hi) continue;
    const int jlo = s_first[lk_lo], jhi = s_first[lk_hi + 1];
    // this warp's items: index congruent to the warp
    for (int j0 = jlo + ((warp - jlo) % kWarps + kWarps) % kWarps; j0 < jhi;
         j0 += 2 * kWarps) {
      const bool two = j0 + kWarps < jhi;  // warp-uniform
      float sr[2][LM::NPL], si[2][LM::NPL], kf[2];
      float kv[2][LM::RS == 1 ? AW : 1];
      const float2 *base[2][LM::NPL];
      const float *kjs[2];
      int lvs[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int jj = (u == 1 && two) ? j0 + kWarps : j0;
        const float *kj = kc + jj * KS;
        kjs[u] = kj;
        const uint32_t loc = __float_as_uint(kj[0]);
        const int lu = (int)(loc & 0xffu);
        lvs[u] = (int)((loc >> 8) & 0xffu);
        const int aw = k - (kbase + (int)((loc >> 16) & 0xffu));  // in [0, wk) here
        kf[u] = kj[4 + 2 * AW + aw] * kj[4 + lm.a];               // kw(aw) ku(a), signed
        if constexpr (LM::RS == 1) {
#pragma unroll
          for (int q = 0; q < AW; q += 4) {
            const float4 t = *reinterpret_cast<const float4 *>(kj + 4 + AW + q);
            kv[u][q] = t.x;
            kv[u][q + 1] = t.y;
            kv[u][q + 2] = t.z;
            kv[u][q + 3] = t.w;
          }
        }
        const int col = s_col[lu + (lane_in ? lm.a : 0)];
#pragma unroll
        for (int i = 0; i < LM::NPL; ++i) {
          base[u][i] = gplane + lm.pol(i) * plane + col;
          sr[u][i] = 0.f;
          si[u][i] = 0.f;
        }
      }
#pragma unroll
      for (int r = 0; r < kMaxRows; ++r) {
        if (LM::RS == 1 && r >= W) break;  // warp-uniform
        const int b = lm.r0 + r * LM::RS;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          if (u == 1 && !two) break;  // warp-uniform
          if (b < W && lane_in) {
            float kvb;
            if constexpr (LM::RS == 1)
              kvb = kv[u][r];
            else
              kvb = kjs[u][4 + AW + b];
            const int ro = s_rowoff[lvs[u] + b];
#pragma unroll
            for (int i = 0; i < LM::NPL; ++i) {
              const float2 v = __ldg(base[u][i] + ro);
              sr[u][i] += kvb * v.x;
              si[u][i] += kvb * v.y;
            }
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (u == 1 && !two) break;  // warp-uniform
        const int jj = u == 1 ? j0 + kWarps : j0;
#pragma unroll
        for (int i = 0; i < LM::NPL; ++i) {
          float xr = sr[u][i] * kf[u], xi = si[u][i] * kf[u];
#pragma unroll
          for (int o = 1; o < AW; o <<= 1) {
            xr += __shfl_xor_sync(0xffffffffu, xr, o);
            xi += __shfl_xor_sync(0xffffffffu, xi, o);
          }
          if (NP < LM::G) {  // groups sharing a pol hold different rows
#pragma unroll
            for (int o = AW * NP; o < 32; o <<= 1) {
              xr += __shfl_xor_sync(0xffffffffu, xr, o);
              xi += __shfl_xor_sync(0xffffffffu, xi, o);
            }
          }
          if (lm.a == 0 && lm.r0 == 0) {  // only this warp touches item jj
            float2 &s = sacc[jj * NP + lm.pol(i)];
            s.x += xr;
            s.y += xi;
          }
        }
      }
    }
  }
  __syncthreads();  // every item's sums complete
  for (int jj = threadIdx.x; jj < n; jj += kThreads) {
    const ItemF it = items[ch.begin + jj];
    const int k0 = kbase + (int)((it.loc >> 16) & 0xffu);
    if (!(k0 + wk > b0 && k0 < b0 + nb)) continue;
    float2 v[NP];
    // a mirrored item (at -uvw) predicts the conjugate
    const float conj_sign = (it.loc & kLocFlip) ? -1.f : 1.f;
#pragma unroll
    for (int p = 0; p < NP; ++p) {  // multiply by conj(ph) = exp(+2 pi i w tc)
      const float2 a = sacc[jj * NP + p];
      v[p].x = a.x * it.ph.x + a.y * it.ph.y;
      v[p].y = (a.y * it.ph.x - a.x * it.ph.y) * conj_sign;
    }
    const size_t vbase = (size_t)it.idx * npv;
    const bool first = k0 >= b0;
    for (int q = 0; q < npv; ++q) {
      float2 o = v[0];
      if (pm.identity) {
#pragma unroll
        for (int p = 1; p < NP; ++p)
          if (p == (q < NP ? q : NP - 1)) o = v[p];
      } else {
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const float mr = pm.fre[q * pm.nin + p], mi = pm.fim[q * pm.nin + p];
          re += mr * v[p].x - mi * v[p].y;
          im += mr * v[p].y + mi * v[p].x;
        }
        o = make_float2(re, im);
      }
      if (wgt) {
        const float w = wgt[vbase + q];
        o.x *= w;
        o.y *= w;
      }
      if (first) {
        vis[vbase + q] = o;
      } else {
        float2 prev = vis[vbase + q];
        prev.x += o.x;
        prev.y += o.y;
        vis[vbase + q] = prev;
      }
    }
  }
}

// CTAs per SM the warp degridders are compiled for: few enough that the
// CTAs' tiles of one plane fit L1 beside their shared memory.
constexpr int kDegridWarpBlocks = 3;

// Dynamic shared memory of the warp degridder: the item cache, then the
// per-item sums.
__host__ __device__ constexpr size_t degrid_warp_smem(int AW, int NP) {
  return (size_t)kChunkItems * (kcache_stride(AW) * sizeof(float) + NP * sizeof(float2));
}

template <int NP, int AW>
__global__ void __launch_bounds__(kThreads, kDegridWarpBlocks)
    k_degrid_warp(const Geom g, const ItemF *__restrict__ items, const Chunk *__restrict__ chunks,
                  const uint32_t *__restrict__ chunk_off, int b0, int nb,
                  const float2 *__restrict__ grid, float2 *__restrict__ vis, int npv,
                  const float *__restrict__ wgt, const PolMat pm, const RowPerm rp,
                  uint32_t *__restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *kc = reinterpret_cast<float *>(smem_raw);                               // item cache
  float2 *sacc = reinterpret_cast<float2 *>(kc + kChunkItems * kcache_stride(AW));  // sums
  __shared__ int s_first[kMaxSlab + 1], s_rowoff[kMaxSubSide], s_col[kMaxSubSide];
  __shared__ uint32_t s_ci;
  const int ntiles = g.ntu * g.ntv;
  const int wk = g.do_w ? g.W : 1;
  const int lo = b0 - (g.S + wk - 2);
  const int s_lo = lo <= 0 ? 0 : (lo + g.S - 1) / g.S;
  const int s_hi = min(g.nslabs - 1, (b0 + nb - 1) / g.S);
  const uint32_t c_begin = chunk_off[(int64_t)s_lo * ntiles];
  const uint32_t c_end = chunk_off[(int64_t)(s_hi + 1) * ntiles];
  for (;;) {
    if (threadIdx.x == 0) s_ci = c_begin + atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t ci = s_ci;
    __syncthreads();  // every thread has read s_ci (and the last chunk's tables)
    if (ci >= c_end) break;
    degrid_warp_chunk<NP, AW>(g, items, chunks[ci], b0, nb, grid, vis, npv, wgt, pm, rp, kc,
                              sacc, s_first, s_rowoff, s_col);
  }
}

// Many plans' degridding in one persistent launch (FP32 form, one lane
// width): the work queue is the concatenation of every job's chunk range,
// as in k_grid_jobs; each CTA takes the next index from one atomic counter
// and degrids that chunk of its job into the job's visibilities.
template <int NP, int AW>
__global__ void __launch_bounds__(kThreads, kDegridWarpBlocks)
    k_degrid_warp_jobs(const __grid_constant__ GridJobs jobs, const PolMat pm,
                       uint32_t *__restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *kc = reinterpret_cast<float *>(smem_raw);
  float2 *sacc = reinterpret_cast<float2 *>(kc + kChunkItems * kcache_stride(AW));
  __shared__ int s_first[kMaxSlab + 1], s_rowoff[kMaxSubSide], s_col[kMaxSubSide];
  __shared__ uint32_t s_wbeg[kMaxJobs + 1], s_cbeg[kMaxJobs];
  __shared__ uint32_t s_w;
  __shared__ int s_j;
  if (threadIdx.x == 0) {
    uint32_t w = 0;
    for (int j = 0; j < jobs.n; ++j) {
      const GridJob &jb = jobs.job[j];
      const Geom &g = jb.g;
      const int ntiles = g.ntu * g.ntv;
      const int wk = g.do_w ? g.W : 1;
      const int lo = jb.b0 - (g.S + wk - 2);
      const int s_lo = lo <= 0 ? 0 : (lo + g.S - 1) / g.S;
      const int s_hi = min(g.nslabs - 1, (jb.b0 + jb.nb - 1) / g.S);
      const uint32_t c0 = jb.chunk_off[(int64_t)s_lo * ntiles];
      const uint32_t c1 = jb.chunk_off[(int64_t)(s_hi + 1) * ntiles];
      s_wbeg[j] = w;
      s_cbeg[j] = c0;
      w += c1 > c0 ? c1 - c0 : 0u;
    }
    s_wbeg[jobs.n] = w;
  }
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
    const int j = s_j;
    __syncthreads();  // every thread has read s_w, s_j
    if (w >= total) break;
    const GridJob &jb = jobs.job[j];
    const uint32_t ci = s_cbeg[j] + (w - s_wbeg[j]);
    degrid_warp_chunk<NP, AW>(jb.g, reinterpret_cast<const ItemF *>(jb.items), jb.chunks[ci],
                              jb.b0, jb.nb, reinterpret_cast<const float2 *>(jb.grid),
                              reinterpret_cast<float2 *>(jb.vis), jb.npv, jb.wgt, pm, jb.rp, kc,
                              sacc, s_first, s_rowoff, s_col);
  }
}

size_t degrid_warp_smem_bytes(const gb_plan *p) {
  return degrid_warp_smem(group_lanes(p->g.W), p->g.NP);
}

// Shared-memory carveout (percent of the SM's maximum) that holds `per_sm`
// CTAs of `smem` bytes and leaves the rest of the unified array to L1.
static int degrid_carveout(size_t smem, int per_sm) {
  int dev = 0, max_smem = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  if (max_smem <= 0) return -1;
  const size_t need = (size_t)per_sm * (smem + 3072);  // + static and reserved shared memory
  const int pct = (int)((need * 100 + max_smem - 1) / max_smem);
  return pct > 100 ? 100 : pct;
}

template <int NP, int AW>
static int setup_degrid_warp_aw(gb_plan *p) {
  const size_t smem = degrid_warp_smem_bytes(p);
  auto k = k_degrid_warp<NP, AW>;
  GB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int pct = degrid_carveout(smem, kDegridWarpBlocks);
  if (pct > 0) GB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem));
  if (per_sm < 1) {
    set_error("k_degrid_warp cannot launch with %zu bytes of shared memory", smem);
    return GB_ERR_INVALID_ARG;
  }
  p->degrid_blocks = per_sm * p->num_sms;
  return GB_OK;
}

template <int NP>
static int setup_degrid_warp(gb_plan *p) {
  return group_lanes(p->g.W) == 8 ? setup_degrid_warp_aw<NP, 8>(p)
                                  : setup_degrid_warp_aw<NP, 16>(p);
}

// The predict driver in steps (gb_batch.cu interleaves them across plans):
// begin (corrected image), then per w-plane batch bi: transform (screens +
// 2-D transform into the batch buffer), degrid.
template <typename R, int NP>
static int pred_begin_impl(gb_plan *p, const void *dirty, int layout, cudaStream_t s) {
  const Geom &g = p->g;
  R *img = reinterpret_cast<R *>(p->ws + p->off_temp + p->c_img);
  uint32_t *counters = p->at<uint32_t>(p->off_counters) + p->nbatches;
  GB_CUDA(cudaMemsetAsync(counters, 0, 4 * (size_t)p->nbatches, s));
  dim3 fb((g.nx + 31) / 32, (g.ny + 31) / 32, NP);
  const double npix = (double)g.nx * g.ny;
  ProfScope ps(kProfPrepImage, s, 3.0 * sizeof(R) * NP * npix);
  k_prep_image<R><<<fb, dim3(32, 8), 0, s>>>(g, reinterpret_cast<const R *>(dirty), layout,
                                             p->at<R>(p->off_corr), img);
  GB_LAUNCH_CHECK("k_prep_image");
  return GB_OK;
}

template <typename R, int NP>
static int pred_transform_impl(gb_plan *p, int bi, cudaStream_t s) {
  using C = typename Traits<R>::C;
  const Geom &g = p->g;
  char *tmp = p->ws + p->off_temp;
  C *grid = reinterpret_cast<C *>(tmp + p->c_grid);
  R *img = reinterpret_cast<R *>(tmp + p->c_img);
  const int b0 = bi * g.B, nb = std::min(g.B, g.nplanes - b0);
  const int64_t plane = (int64_t)g.ngx * g.ngy;
  const double gbytes = (double)sizeof(C) * nb * NP * (double)plane;
  const double npix = (double)g.nx * g.ny;
  bool cols = false;
  if constexpr (std::is_same<R, float>::value) {
    if (p->col_fft) {  // screen + columns now, rows below
      const int rc = run_cols_predict(p, img, b0, nb, grid, s);
      if (rc) return rc;
      cols = true;
    }
  }
  if (!cols) {
    const unsigned cell_blocks = (unsigned)std::min<int64_t>((plane + kThreads - 1) / kThreads,
                                                             (int64_t)p->num_sms * 32);
    ProfScope ps(kProfScreenPad, s, gbytes + sizeof(R) * NP * npix);
    k_screen_pad<R, NP><<<cell_blocks, kThreads, 0, s>>>(g, img, p->at<double>(p->off_tprime),
                                                         b0, nb, grid);
    GB_LAUNCH_CHECK("k_screen_pad");
  }
  if (p->row_fft) {
    // image half in, row out
    ProfScope ps(kProfRowsFwd, s, 1.5 * p->used_rows(b0, nb) * gbytes);
    return run_rows(p, grid, b0, nb, -1, s);
  }
  ProfScope ps(kProfFftFwd, s, 2.0 * gbytes);
  return run_fft(p, nb, grid, CUFFT_FORWARD, s);
}

// Algorithmic bytes and updates of degridding batch bi (profiling): items
// read, their vis written once; the grid cells they reach read once (the
// cells of the (plane, tile) pairs reached, else the rows).
template <typename R, int NP>
static void degrid_counts(const gb_plan *p, int bi, int npv, bool wgt, double *bytes,
                          double *updates) {
  using C = typename Traits<R>::C;
  using Item = typename Traits<R>::Item;
  const Geom &g = p->g;
  const int b0 = bi * g.B, nb = std::min(g.B, g.nplanes - b0);
  const double gbytes = (double)sizeof(C) * nb * NP * (double)g.ngx * g.ngy;
  const double cells = p->touched_cells(b0, nb);
  const double gread = cells > 0.0 ? cells * NP * sizeof(C) : p->used_rows(b0, nb) * gbytes;
  *bytes = (double)p->batch_items(b0, nb) *
               (sizeof(Item) + npv * sizeof(C) + (wgt ? npv * sizeof(R) : 0.0)) + gread;
  *updates = p->item_planes(b0, nb) * g.W * g.W * NP;
}

template <typename R, int NP>
static int pred_degrid_impl(gb_plan *p, int bi, const void *wgt, const PolMat &pm, int npv,
                            void *vis, cudaStream_t s) {
  using C = typename Traits<R>::C;
  using Item = typename Traits<R>::Item;
  const Geom &g = p->g;
  C *grid = reinterpret_cast<C *>(p->ws + p->off_temp + p->c_grid);
  uint32_t *counters = p->at<uint32_t>(p->off_counters) + p->nbatches;
  const Item *items = p->at<Item>(p->off_items);
  const Chunk *chunks = p->at<Chunk>(p->off_chunks);
  const uint32_t *chunk_off = p->at<uint32_t>(p->off_chunk_off);
  const int b0 = bi * g.B, nb = std::min(g.B, g.nplanes - b0);
  const RowPerm rperm = row_perm(p);
  C *vis_c = reinterpret_cast<C *>(vis);
  double bytes = 0.0, updates = 0.0;
  if (prof_on()) degrid_counts<R, NP>(p, bi, npv, wgt != nullptr, &bytes, &updates);
  ProfScope ps(kProfDegrid, s, bytes, updates);
  if constexpr (std::is_same<R, float>::value) {
    const size_t smem = degrid_warp_smem_bytes(p);
    if (group_lanes(g.W) == 8)
      k_degrid_warp<NP, 8><<<p->degrid_blocks, kThreads, smem, s>>>(
          g, items, chunks, chunk_off, b0, nb, grid, vis_c, npv, reinterpret_cast<const R *>(wgt),
          pm, rperm, counters + bi);
    else
      k_degrid_warp<NP, 16><<<p->degrid_blocks, kThreads, smem, s>>>(
          g, items, chunks, chunk_off, b0, nb, grid, vis_c, npv, reinterpret_cast<const R *>(wgt),
          pm, rperm, counters + bi);
  } else {
    const size_t smem = tile_smem_bytes(p);
    if (group_lanes(g.W) == 8)
      k_degrid<R, NP, 8><<<p->degrid_blocks, kThreads, smem, s>>>(
          g, items, chunks, chunk_off, b0, nb, grid, vis_c, npv, reinterpret_cast<const R *>(wgt),
          pm, rperm, counters + bi);
    else
      k_degrid<R, NP, 16><<<p->degrid_blocks, kThreads, smem, s>>>(
          g, items, chunks, chunk_off, b0, nb, grid, vis_c, npv, reinterpret_cast<const R *>(wgt),
          pm, rperm, counters + bi);
  }
  GB_LAUNCH_CHECK("k_degrid");
  return GB_OK;
}

template <typename R, int NP>
static int dirty2ms_impl(gb_plan *p, const void *dirty, int layout, const void *wgt,
                         const PolMat &pm, int npv, void *vis, cudaStream_t s) {
  int rc = pred_begin_impl<R, NP>(p, dirty, layout, s);
  for (int bi = 0; !rc && bi < p->nbatches; ++bi) {
    rc = pred_transform_impl<R, NP>(p, bi, s);
    if (!rc) rc = pred_degrid_impl<R, NP>(p, bi, wgt, pm, npv, vis, s);
  }
  return rc;
}

#define GB_PRED_DISPATCH(p, CALL)                    \
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

int pred_begin(gb_plan *p, const void *dirty, int layout, cudaStream_t s) {
  GB_PRED_DISPATCH(p, (pred_begin_impl<R, NP>(p, dirty, layout, s)));
}
int pred_transform(gb_plan *p, int bi, cudaStream_t s) {
  GB_PRED_DISPATCH(p, (pred_transform_impl<R, NP>(p, bi, s)));
}

// Fill one job of a multi-plan degridding launch from a bound FP32 plan
// whose batch bi has been transformed.
int degrid_job(gb_plan *p, int bi, void *vis, int npv, GridJob &jb) {
  if (p->precision != GB_FP32 || !p->bound || bi < 0 || bi >= p->nbatches) {
    set_error("degrid_job: needs a bound FP32 plan and a batch index in range");
    return GB_ERR_INVALID_ARG;
  }
  char *tmp = p->ws + p->off_temp;
  jb.g = p->g;
  jb.items = p->at<ItemF>(p->off_items);
  jb.cvis = nullptr;
  jb.chunks = p->at<Chunk>(p->off_chunks);
  jb.chunk_off = p->at<uint32_t>(p->off_chunk_off);
  jb.grid = tmp + p->c_grid;
  jb.b0 = bi * p->g.B;
  jb.nb = std::min(p->g.B, p->g.nplanes - jb.b0);
  jb.vis = vis;
  jb.npv = npv;
  jb.pad = 0;
  jb.wgt = nullptr;
  jb.rp = row_perm(p);
  return GB_OK;
}

void degrid_job_counts(const gb_plan *p, int bi, int npv, double *bytes, double *updates) {
  *bytes = 0.0;
  *updates = 0.0;
  if (!prof_on()) return;
  switch (p->g.NP) {
    case 1: degrid_counts<float, 1>(p, bi, npv, false, bytes, updates); break;
    case 2: degrid_counts<float, 2>(p, bi, npv, false, bytes, updates); break;
    default: degrid_counts<float, 4>(p, bi, npv, false, bytes, updates); break;
  }
}

// One launch over `jobs` (all of one NP and support W, unit weights, one pol
// matrix); `counter` must be zero.
int launch_degrid_jobs(const GridJobs &jobs, const PolMat &pm, int num_sms, uint32_t *counter,
                       double bytes, double updates, cudaStream_t s) {
  if (jobs.n < 1 || jobs.n > kMaxJobs) {
    set_error("launch_degrid_jobs: %d jobs (1..%d)", jobs.n, kMaxJobs);
    return GB_ERR_INVALID_ARG;
  }
  const int NP = jobs.job[0].g.NP, AW = group_lanes(jobs.job[0].g.W);
  for (int j = 0; j < jobs.n; ++j) {
    const Geom &g = jobs.job[j].g;
    if (g.NP != NP || group_lanes(g.W) != AW) {
      set_error("launch_degrid_jobs: jobs of one launch share NP and the lane width");
      return GB_ERR_INVALID_ARG;
    }
  }
  const size_t smem = degrid_warp_smem(AW, NP);
  ProfScope ps(kProfDegrid, s, bytes, updates);
#define GB_DJ(NPV, AWV)                                                                       \
  {                                                                                           \
    auto k = k_degrid_warp_jobs<NPV, AWV>;                                                    \
    GB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));  \
    const int pct = degrid_carveout(smem, kDegridWarpBlocks);                                 \
    if (pct > 0)                                                                              \
      GB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, pct));  \
    int per_sm = 0;                                                                           \
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem));       \
    if (per_sm < 1) {                                                                         \
      set_error("k_degrid_warp_jobs cannot launch with %zu bytes of shared memory", smem);   \
      return GB_ERR_INVALID_ARG;                                                              \
    }                                                                                         \
    k<<<per_sm * num_sms, kThreads, smem, s>>>(jobs, pm, counter);                           \
  }
  if (AW == 8) {
    if (NP == 1) GB_DJ(1, 8) else if (NP == 2) GB_DJ(2, 8) else GB_DJ(4, 8)
  } else {
    if (NP == 1) GB_DJ(1, 16) else if (NP == 2) GB_DJ(2, 16) else GB_DJ(4, 16)
  }
#undef GB_DJ
  GB_LAUNCH_CHECK("k_degrid_warp_jobs");
  return GB_OK;
}

int run_dirty2ms(gb_plan *p, const void *dirty, int layout, const void *wgt, const PolMat &pm,
                 int npv, void *vis, cudaStream_t s) {
#define GB_CASE(R, NP) return dirty2ms_impl<R, NP>(p, dirty, layout, wgt, pm, npv, vis, s)
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
static int setup_degrid_aw(gb_plan *p) {
  const size_t smem = tile_smem_bytes(p);
  GB_CUDA(cudaFuncSetAttribute(k_degrid<R, NP, AW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_degrid<R, NP, AW>, kThreads,
                                                        smem));
  if (per_sm < 1) {
    set_error("k_degrid cannot launch with %zu bytes of shared memory", smem);
    return GB_ERR_INVALID_ARG;
  }
  p->degrid_blocks = per_sm * p->num_sms;
  return GB_OK;
}

template <typename R, int NP>
static int setup_degrid_impl(gb_plan *p) {
  if constexpr (std::is_same<R, float>::value) return setup_degrid_warp<NP>(p);
  return group_lanes(p->g.W) == 8 ? setup_degrid_aw<R, NP, 8>(p)
                                  : setup_degrid_aw<R, NP, 16>(p);
}

int setup_tile_kernels(gb_plan *p) {
  int rc = setup_grid_kernels(p);
  if (rc) return rc;
  if (p->precision == GB_FP64) {
    switch (p->g.NP) {
      case 1: return setup_degrid_impl<double, 1>(p);
      case 2: return setup_degrid_impl<double, 2>(p);
      default: return setup_degrid_impl<double, 4>(p);
    }
  }
  switch (p->g.NP) {
    case 1: return setup_degrid_impl<float, 1>(p);
    case 2: return setup_degrid_impl<float, 2>(p);
    default: return setup_degrid_impl<float, 4>(p);
  }
}

}  // namespace gb
