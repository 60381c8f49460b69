// Predict (dirty2ms): model image -> visibilities.
//
// Per call:   k_prep_image  image * correction, into [pol][y][x] order.
// Per batch of w-planes:
//             k_screen_pad  every grid cell of every plane in the batch is
//                           written once: the central block gets
//                           image * exp(+2 pi i w_k (n-1-tc)), the rest 0
//                           (no separate memset pass).
//             cuFFT         2-D c2c, e^{-2 pi i}
//             k_degrid      one CTA per work chunk: the tile's sub-grid of
//                           each plane is staged in shared memory from
//                           coalesced 16-byte grid rows; each warp walks its
//                           items, each lane sums a slice of the W x W
//                           support and the partial sums are reduced with
//                           warp shuffles; lane i keeps item i's running
//                           sum over planes.  The epilogue rotates back by
//                           exp(+2 pi i w tc), applies the pol-frame matrix
//                           and weights and writes (first batch of the
//                           item) or accumulates (later batches) in place.
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

// float2 elements from one staged row to the next in k_degrid_lane: SW
// cells padded to an odd count, plus one 16-byte unit for NP = 4.
__host__ __device__ constexpr int lane_row(int NP, int SW) {
  return (SW | 1) * NP + (NP == 4 ? 2 : 0);
}

// Pols summed per staging pass of k_degrid_lane: two for NP = 4 (half the
// staging and per-thread sums, so more CTAs fit an SM), else all.
__host__ __device__ constexpr int degrid_pass_pols(int NP) { return NP == 4 ? 2 : NP; }

// FP32 degridder, one item per thread.  A CTA takes a chunk (up to 256
// items of one bucket); thread i owns item i: its u and v kernel values
// (with the checkerboard sign (-1)^(p+q) folded in) stay in registers for
// all planes, and for every plane the thread sums its whole W x W footprint
// from the plane's staged sub-grid ([SW][pitch][NP] complex, a cell's pols
// contiguous), double-buffered with cp.async so plane k + 1 streams in
// while plane k is summed.  Staged rows are lane_row(NP, SW) float2 apart:
// an odd number of 16-byte units for NP = 4 (whose cells are two 16-byte
// units), so one load instruction's 32 cells spread over all eight 16-byte
// bank groups instead of the four of one parity.
// Per item-plane that is W^2 NP shared loads and 2 W^2 NP FMAs with no
// cross-lane reduction, against the warp-per-item map of k_degrid.
// Degrid one work chunk (up to kChunkItems items of one bucket, thread i
// owning item i) over the planes [b0, b0 + nb) of `grid` into vis.  stage /
// skv: the block's shared staging buffers (2 x [SW][rowf2] float2, then
// [WT][kThreads] floats).  Every thread of the block calls it; it ends with
// the staging buffers free.
template <int NP, int WT>
__device__ __forceinline__ void degrid_lane_chunk(
    const Geom &g, const ItemF *__restrict__ items, const Chunk ch, int b0, int nb,
    const float2 *__restrict__ grid, float2 *__restrict__ vis, int npv,
    const float *__restrict__ wgt, const PolMat &pm, const RowPerm &rp, float2 *stage,
    float *skv, int *s_rowoff, int *s_col) {
  constexpr int PP = degrid_pass_pols(NP);
  const int T = g.T;
  const int SW = T + WT - 1, rowf2 = lane_row(PP, SW), pstride = SW * rowf2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  (void)lane;
  const float scale_u = 2.f / (float)WT;
  const float beta = (float)g.beta;
  const int ntiles = g.ntu * g.ntv;
  const int64_t plane = (int64_t)g.ngx * g.ngy;
  const int wk = g.do_w ? WT : 1;
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
    const int k_hi = min(min(kbase + lk_last + WT, g.nplanes), b0 + nb);
    if (k_lo >= k_hi) return;  // (block-uniform) no item reaches this batch's planes
    const int n = (int)(ch.end - ch.begin);
    const bool direct = n * WT * WT < SW * SW;
    const bool has = (int)threadIdx.x < n;
    ItemF it = items[ch.begin + (has ? threadIdx.x : 0)];
    const int lu = (int)(it.loc & 0xffu), lv = (int)((it.loc >> 8) & 0xffu);
    const int k0 = kbase + (int)((it.loc >> 16) & 0xffu);
    const int tpar = ((tu + tv) * T) & 1;  // checkerboard parity of the tile origin
    float ku[WT];
#pragma unroll
    for (int a = 0; a < WT; ++a) {
      const float x = es_kernel(((float)a - it.du) * scale_u, beta);
      const float y = es_kernel(((float)a - it.dv) * scale_u, beta);
      ku[a] = ((lu + a + tpar) & 1) ? -x : x;
      skv[a * kThreads + threadIdx.x] = ((lv + a) & 1) ? -y : y;
    }
    float2 acc[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[p] = make_float2(0.f, 0.f);
    // the sub-grid's grid rows (physical row x ngx, in the row order of the
    // grid) and columns, wrapped once per chunk for every staged plane
    if (!direct) {
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
      __syncthreads();
    }
    // the pols in passes of PP: each pass stages its pols' sub-grids only,
    // which halves the staging buffers and the per-thread sums for NP = 4
    // (unrolled: acc stays in registers)
#pragma unroll
    for (int pb = 0; pb < NP; pb += PP) {
      // raw sub-grid of plane k (pols pb .. pb + PP) -> dst, one cp.async
      // commit group per thread
      auto stage_plane = [&](int k, float2 *dst) {
        const float2 *gp = grid + ((int64_t)(k - b0) * NP + pb) * plane;
        static_assert(PP <= 2, "one or two pols per staging pass");
        for (int r = warp; r < PP * SW; r += kWarps) {
          const int pol = r >= SW ? 1 : 0, y = r - pol * SW;
          const float2 *src = gp + pol * plane + s_rowoff[y];
          float2 *d = dst + y * rowf2 + pol;
          for (int x = lane; x < SW; x += 32) cp_async8(d + x * PP, src + s_col[x], true);
        }
        cp_async_commit();
      };
      if (!direct && k_lo < k_hi) stage_plane(k_lo, stage);
      for (int k = k_lo; k < k_hi; ++k) {
        const float2 *gp = grid + ((int64_t)(k - b0) * NP + pb) * plane;
        const float2 *sg = stage + ((k - k_lo) & 1) * pstride;
        if (!direct) {
          // plane k + 1 goes to the other buffer (consumed in iteration k - 1,
          // released by that iteration's closing barrier)
          if (k + 1 < k_hi) {
            stage_plane(k + 1, stage + ((k + 1 - k_lo) & 1) * pstride);
            cp_async_wait1();
          } else {
            cp_async_wait0();
          }
          __syncthreads();  // plane k staged by every thread
        }
        const int aw = k - k0;
        if (has && aw >= 0 && aw < wk) {
          const float fw = g.do_w ? es_kernel(((float)aw - it.dwf) * scale_u, beta) : 1.f;
          float2 sum[PP];
#pragma unroll
          for (int p = 0; p < PP; ++p) sum[p] = make_float2(0.f, 0.f);
#pragma unroll 1
          for (int b = 0; b < WT; ++b) {
            float2 rs[PP];
#pragma unroll
            for (int p = 0; p < PP; ++p) rs[p] = make_float2(0.f, 0.f);
            if (direct) {
              int q = tv * T + lv + b;
              while (q >= g.ngy) q -= g.ngy;
              const float2 *row = gp + (int64_t)rp.row(q) * g.ngx;
#pragma unroll
              for (int a = 0; a < WT; ++a) {
                int pc = tu * T + lu + a;
                while (pc >= g.ngx) pc -= g.ngx;
#pragma unroll
                for (int p = 0; p < PP; ++p) {
                  const float2 v = row[p * plane + pc];
                  rs[p].x += ku[a] * v.x;
                  rs[p].y += ku[a] * v.y;
                }
              }
            } else {
              // a cell's PP values are contiguous: 16-byte loads of two pols
              const float2 *row = sg + (lv + b) * rowf2 + lu * PP;
#pragma unroll
              for (int a = 0; a < WT; ++a) {
                if constexpr (PP == 1) {
                  const float2 v = row[a];
                  rs[0].x += ku[a] * v.x;
                  rs[0].y += ku[a] * v.y;
                } else {
#pragma unroll
                  for (int pp = 0; pp < PP / 2; ++pp) {
                    const float4 v = *reinterpret_cast<const float4 *>(row + a * PP + 2 * pp);
                    rs[2 * pp].x += ku[a] * v.x;
                    rs[2 * pp].y += ku[a] * v.y;
                    rs[2 * pp + 1].x += ku[a] * v.z;
                    rs[2 * pp + 1].y += ku[a] * v.w;
                  }
                }
              }
            }
            const float kvb = skv[b * kThreads + threadIdx.x];
#pragma unroll
            for (int p = 0; p < PP; ++p) {
              sum[p].x += kvb * rs[p].x;
              sum[p].y += kvb * rs[p].y;
            }
          }
#pragma unroll
          for (int p = 0; p < PP; ++p) {
            acc[pb + p].x += fw * sum[p].x;
            acc[pb + p].y += fw * sum[p].y;
          }
        }
        if (!direct) __syncthreads();  // buffer consumed before it is refilled
      }
    }
    if (has && k0 + wk > b0 && k0 < b0 + nb) {
      float2 v[NP];
      // a mirrored item (at -uvw) predicts the conjugate
      const float conj_sign = (it.loc & kLocFlip) ? -1.f : 1.f;
#pragma unroll
      for (int p = 0; p < NP; ++p) {  // multiply by conj(ph) = exp(+2 pi i w tc)
        v[p].x = acc[p].x * it.ph.x + acc[p].y * it.ph.y;
        v[p].y = (acc[p].y * it.ph.x - acc[p].x * it.ph.y) * conj_sign;
      }
      const size_t base = (size_t)it.idx * npv;
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
          const float w = wgt[base + q];
          o.x *= w;
          o.y *= w;
        }
        if (first) {
          vis[base + q] = o;
        } else {
          float2 prev = vis[base + q];
          prev.x += o.x;
          prev.y += o.y;
          vis[base + q] = prev;
        }
      }
    }
  }
}

// CTAs per SM the lane degridders are compiled for (registers <= 80).
constexpr int kDegridLaneBlocks = 3;

template <int NP, int WT>
__global__ void __launch_bounds__(kThreads, kDegridLaneBlocks)
    k_degrid_lane(const Geom g, const ItemF *__restrict__ items, const Chunk *__restrict__ chunks,
                  const uint32_t *__restrict__ chunk_off, int b0, int nb,
                  const float2 *__restrict__ grid, float2 *__restrict__ vis, int npv,
                  const float *__restrict__ wgt, const PolMat pm, const RowPerm rp,
                  uint32_t *__restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int SW = g.T + WT - 1, pstride = SW * lane_row(degrid_pass_pols(NP), SW);
  float2 *stage = reinterpret_cast<float2 *>(smem_raw);          // 2 x [SW][rowf2]
  float *skv = reinterpret_cast<float *>(stage + 2 * pstride);   // [WT][kThreads]: own kv
  __shared__ int s_rowoff[kMaxSubSide], s_col[kMaxSubSide];
  const int ntiles = g.ntu * g.ntv;
  const int lo = b0 - (g.S + WT - 2);
  const int s_lo = lo <= 0 ? 0 : (lo + g.S - 1) / g.S;
  const int s_hi = min(g.nslabs - 1, (b0 + nb - 1) / g.S);
  const uint32_t c_begin = chunk_off[(int64_t)s_lo * ntiles];
  const uint32_t c_end = chunk_off[(int64_t)(s_hi + 1) * ntiles];
  __shared__ uint32_t s_ci;
  for (;;) {
    if (threadIdx.x == 0) s_ci = c_begin + atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t ci = s_ci;
    __syncthreads();  // every thread has read s_ci
    if (ci >= c_end) break;
    degrid_lane_chunk<NP, WT>(g, items, chunks[ci], b0, nb, grid, vis, npv, wgt, pm, rp, stage,
                              skv, s_rowoff, s_col);
  }
}

// Many plans' degridding in one persistent launch (FP32 form, one support
// WT): the work queue is the concatenation of every job's chunk range, as
// in k_grid_jobs; each CTA takes the next index from one atomic counter and
// degrids that chunk of its job into the job's visibilities.
template <int NP, int WT>
__global__ void __launch_bounds__(kThreads, kDegridLaneBlocks)
    k_degrid_lane_jobs(const __grid_constant__ GridJobs jobs, const PolMat pm,
                       uint32_t *__restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint32_t s_wbeg[kMaxJobs + 1], s_cbeg[kMaxJobs];
  __shared__ uint32_t s_w;
  __shared__ int s_j;
  int pstride_max = 0;
  for (int j = 0; j < jobs.n; ++j) {
    const int SW = jobs.job[j].g.T + WT - 1;
    pstride_max = max(pstride_max, SW * lane_row(degrid_pass_pols(NP), SW));
  }
  float2 *stage = reinterpret_cast<float2 *>(smem_raw);
  float *skv = reinterpret_cast<float *>(stage + 2 * pstride_max);
  __shared__ int s_rowoff[kMaxSubSide], s_col[kMaxSubSide];
  if (threadIdx.x == 0) {
    uint32_t w = 0;
    for (int j = 0; j < jobs.n; ++j) {
      const GridJob &jb = jobs.job[j];
      const Geom &g = jb.g;
      const int ntiles = g.ntu * g.ntv;
      const int lo = jb.b0 - (g.S + WT - 2);
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
    degrid_lane_chunk<NP, WT>(jb.g, reinterpret_cast<const ItemF *>(jb.items), jb.chunks[ci],
                              jb.b0, jb.nb, reinterpret_cast<const float2 *>(jb.grid),
                              reinterpret_cast<float2 *>(jb.vis), jb.npv, jb.wgt, pm, jb.rp,
                              stage, skv, s_rowoff, s_col);
  }
}

size_t degrid_lane_smem_bytes(const gb_plan *p) {
  const int SW = p->g.T + p->g.W - 1;
  return (size_t)2 * SW * lane_row(degrid_pass_pols(p->g.NP), SW) * sizeof(float2) +
         (size_t)p->g.W * kThreads * sizeof(float);
}

// Launch k_degrid_lane<NP, W> for the plan's support (4..16).
template <int NP>
static void launch_degrid_lane(const gb_plan *p, unsigned blocks, size_t smem, cudaStream_t s,
                               const ItemF *items, const Chunk *chunks, const uint32_t *chunk_off,
                               int b0, int nb, const float2 *grid, float2 *vis, int npv,
                               const float *wgt, const PolMat &pm, const RowPerm &rp,
                               uint32_t *counter) {
#define GB_DL(WV)                                                                            \
  case WV:                                                                                   \
    k_degrid_lane<NP, WV><<<blocks, kThreads, smem, s>>>(p->g, items, chunks, chunk_off, b0, \
                                                         nb, grid, vis, npv, wgt, pm, rp,    \
                                                         counter);                           \
    break;
  switch (p->g.W) {
    GB_DL(4) GB_DL(5) GB_DL(6) GB_DL(7) GB_DL(8) GB_DL(9) GB_DL(10) GB_DL(11) GB_DL(12)
    GB_DL(13) GB_DL(14) GB_DL(15) GB_DL(16)
    default: break;
  }
#undef GB_DL
}

template <int NP>
static int setup_degrid_lane(gb_plan *p) {
  const size_t smem = degrid_lane_smem_bytes(p);
  int per_sm = 0;
#define GB_DL(WV)                                                                             \
  case WV:                                                                                    \
    GB_CUDA(cudaFuncSetAttribute(k_degrid_lane<NP, WV>,                                       \
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));    \
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_degrid_lane<NP, WV>,     \
                                                          kThreads, smem));                   \
    break;
  switch (p->g.W) {
    GB_DL(4) GB_DL(5) GB_DL(6) GB_DL(7) GB_DL(8) GB_DL(9) GB_DL(10) GB_DL(11) GB_DL(12)
    GB_DL(13) GB_DL(14) GB_DL(15) GB_DL(16)
    default:
      set_error("support %d outside 4..16", p->g.W);
      return GB_ERR_INVALID_ARG;
  }
#undef GB_DL
  if (per_sm < 1) {
    set_error("k_degrid_lane cannot launch with %zu bytes of shared memory", smem);
    return GB_ERR_INVALID_ARG;
  }
  p->degrid_blocks = per_sm * p->num_sms;
  return GB_OK;
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
    launch_degrid_lane<NP>(p, (unsigned)p->degrid_blocks, degrid_lane_smem_bytes(p), s, items,
                           chunks, chunk_off, b0, nb, grid, vis_c, npv,
                           reinterpret_cast<const R *>(wgt), pm, rperm, counters + bi);
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
  const int NP = jobs.job[0].g.NP, W = jobs.job[0].g.W;
  int pstride = 0;
  for (int j = 0; j < jobs.n; ++j) {
    const Geom &g = jobs.job[j].g;
    if (g.NP != NP || g.W != W) {
      set_error("launch_degrid_jobs: jobs of one launch share NP and the support");
      return GB_ERR_INVALID_ARG;
    }
    const int SW = g.T + W - 1;
    pstride = std::max(pstride, SW * lane_row(degrid_pass_pols(NP), SW));
  }
  const size_t smem = (size_t)2 * pstride * sizeof(float2) + (size_t)W * kThreads * sizeof(float);
  ProfScope ps(kProfDegrid, s, bytes, updates);
#define GB_DJ(NPV, WV)                                                                        \
  case WV: {                                                                                  \
    auto k = k_degrid_lane_jobs<NPV, WV>;                                                     \
    GB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));  \
    int per_sm = 0;                                                                           \
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem));       \
    if (per_sm < 1) {                                                                         \
      set_error("k_degrid_lane_jobs cannot launch with %zu bytes of shared memory", smem);   \
      return GB_ERR_INVALID_ARG;                                                              \
    }                                                                                         \
    k<<<per_sm * num_sms, kThreads, smem, s>>>(jobs, pm, counter);                           \
    break;                                                                                    \
  }
#define GB_DJ_NP(NPV)                                                                  \
  switch (W) {                                                                         \
    GB_DJ(NPV, 4) GB_DJ(NPV, 5) GB_DJ(NPV, 6) GB_DJ(NPV, 7) GB_DJ(NPV, 8) GB_DJ(NPV, 9)  \
    GB_DJ(NPV, 10) GB_DJ(NPV, 11) GB_DJ(NPV, 12) GB_DJ(NPV, 13) GB_DJ(NPV, 14)          \
    GB_DJ(NPV, 15) GB_DJ(NPV, 16)                                                        \
    default:                                                                             \
      set_error("support %d outside 4..16", W);                                          \
      return GB_ERR_INVALID_ARG;                                                         \
  }
  if (NP == 1) {
    GB_DJ_NP(1)
  } else if (NP == 2) {
    GB_DJ_NP(2)
  } else {
    GB_DJ_NP(4)
  }
#undef GB_DJ_NP
#undef GB_DJ
  GB_LAUNCH_CHECK("k_degrid_lane_jobs");
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
  if constexpr (std::is_same<R, float>::value) return setup_degrid_lane<NP>(p);
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
