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
        const double tp = tprime[pi];
        for (int j = 0; j < nb; ++j) {
          const double turns = plane_turns(g, b0 + j, tp);
          R s, c;
          sincos_2pi((R)turns, &s, &c);
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
  const int nrow_steps = (W + LM::RS - 1) / LM::RS;
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
    const int k_lo = max(kbase, b0);
    const int k_hi = min(min(kbase + g.S + W - 1, g.nplanes), b0 + nb);
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
        for (int r = 0; r < nrow_steps; ++r) {
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
#pragma unroll
        for (int p = 0; p < NP; ++p) {  // multiply by conj(ph) = exp(+2 pi i w tc)
          v[p].x = ar[p] * it.ph.x + ai[p] * it.ph.y;
          v[p].y = ai[p] * it.ph.x - ar[p] * it.ph.y;
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
              const R mr = (R)pm.re[q * pm.nin + p], mi = (R)pm.im[q * pm.nin + p];
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

template <typename R, int NP>
static int dirty2ms_impl(gb_plan *p, const void *dirty, int layout, const void *wgt,
                         const PolMat &pm, int npv, void *vis, cudaStream_t s) {
  using C = typename Traits<R>::C;
  using Item = typename Traits<R>::Item;
  const Geom &g = p->g;
  char *tmp = p->ws + p->off_temp;
  C *grid = reinterpret_cast<C *>(tmp + p->c_grid);
  R *img = reinterpret_cast<R *>(tmp + p->c_img);
  uint32_t *counters = p->at<uint32_t>(p->off_counters) + p->nbatches;
  const Item *items = p->at<Item>(p->off_items);
  const Chunk *chunks = p->at<Chunk>(p->off_chunks);
  const uint32_t *chunk_off = p->at<uint32_t>(p->off_chunk_off);
  const R *corr = p->at<R>(p->off_corr);
  GB_CUDA(cudaMemsetAsync(counters, 0, 4 * (size_t)p->nbatches, s));
  dim3 fb((g.nx + 31) / 32, (g.ny + 31) / 32, NP);
  const double npix = (double)g.nx * g.ny;
  {
    ProfScope ps(kProfPrepImage, s, 3.0 * sizeof(R) * NP * npix);
    k_prep_image<R><<<fb, dim3(32, 8), 0, s>>>(g, reinterpret_cast<const R *>(dirty), layout,
                                               corr, img);
    GB_LAUNCH_CHECK("k_prep_image");
  }
  const int64_t plane = (int64_t)g.ngx * g.ngy;
  const unsigned cell_blocks = (unsigned)std::min<int64_t>((plane + kThreads - 1) / kThreads,
                                                           (int64_t)p->num_sms * 32);
  const size_t smem = tile_smem_bytes(p);
  const RowPerm rperm = row_perm(p);
  for (int bi = 0; bi < p->nbatches; ++bi) {
    const int b0 = bi * g.B;
    const int nb = std::min(g.B, g.nplanes - b0);
    const double gbytes = (double)sizeof(C) * nb * NP * (double)plane;
    bool cols = false;
    if constexpr (std::is_same<R, float>::value) {
      if (p->col_fft) {  // screen + columns now, rows below
        const int rc = run_cols_predict(p, img, b0, nb, grid, s);
        if (rc) return rc;
        cols = true;
      }
    }
    if (!cols) {
      ProfScope ps(kProfScreenPad, s, gbytes + sizeof(R) * NP * npix);
      k_screen_pad<R, NP><<<cell_blocks, kThreads, 0, s>>>(g, img, p->at<double>(p->off_tprime),
                                                           b0, nb, grid);
      GB_LAUNCH_CHECK("k_screen_pad");
    }
    int rc;
    {
      ProfScope ps(kProfFftFwd, s, 2.0 * gbytes);
      rc = run_fft(p, nb, grid, CUFFT_FORWARD, s);
    }
    if (rc) return rc;
    {
      const double nbi = (double)p->batch_items(b0, nb);
      ProfScope ps(kProfDegrid, s,
                   nbi * (sizeof(Item) + npv * sizeof(C) + (wgt ? npv * sizeof(R) : 0.0)) + gbytes);
      if (group_lanes(g.W) == 8)
        k_degrid<R, NP, 8><<<p->degrid_blocks, kThreads, smem, s>>>(
            g, items, chunks, chunk_off, b0, nb, grid, reinterpret_cast<C *>(vis), npv,
            reinterpret_cast<const R *>(wgt), pm, rperm, counters + bi);
      else
        k_degrid<R, NP, 16><<<p->degrid_blocks, kThreads, smem, s>>>(
            g, items, chunks, chunk_off, b0, nb, grid, reinterpret_cast<C *>(vis), npv,
            reinterpret_cast<const R *>(wgt), pm, rperm, counters + bi);
      GB_LAUNCH_CHECK("k_degrid");
    }
  }
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
