/*
 * FP64 multithreaded CPU restatement of the w-stacking ES gridder
 * (oracle / CPU baseline; test infrastructure only).
 *
 * Same algorithm and conventions as oracle/wgridder.py (which restates the
 * published method behind ducc0.wgridder, the arithmetic that
 * rascil/processing_components/imaging/ng.py:91-120,232-275 calls): per
 * w-plane, spread items onto a sigma-oversampled grid with the ES kernel,
 * (-1)^(p+q) checkerboard, then the caller FFTs the plane and the screen
 * kernels below apply exp(-+2 pi i w_k (n-1-tc)) on the central block.
 *
 * Threading: the grid's rows are cut into bands at least W rows high;
 * items are grouped by the band of their first support row; even bands
 * and odd bands are gridded in two parallel passes, so no two threads
 * ever touch the same grid row at the same time (no atomics).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline double es(double x, double beta) {
  const double t = 1.0 - x * x;
  return t > 0.0 ? exp(beta * (sqrt(t) - 1.0)) : 0.0;
}

/* Grid one plane k.  Items are listed in `order`, grouped by band:
 * band b holds order[band_start[b] .. band_start[b+1]).  grid is
 * [ngy][ngx] complex interleaved and is accumulated into. */
void og_grid_plane(int ngx, int ngy, int W, double beta, int do_w, int k,
                   const int32_t *p0, const int32_t *q0, const int32_t *k0, const double *du,
                   const double *dv, const double *dwf, const double *c /* re,im */,
                   const int64_t *order, const int64_t *band_start, int nbands,
                   double *grid, int nthreads) {
  const double scale = 2.0 / W;
  for (int parity = 0; parity < 2; ++parity) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int b = parity; b < nbands; b += 2) {
      double ku[32], kv[32];
      for (int64_t t = band_start[b]; t < band_start[b + 1]; ++t) {
        const int64_t i = order[t];
        const int aw = k - k0[i];
        if (aw < 0 || aw >= (do_w ? W : 1)) continue;
        const double fw = do_w ? es((aw - dwf[i]) * scale, beta) : 1.0;
        for (int a = 0; a < W; ++a) {
          ku[a] = es((a - du[i]) * scale, beta);
          kv[a] = es((a - dv[i]) * scale, beta);
        }
        const double cr = c[2 * i] * fw, ci = c[2 * i + 1] * fw;
        for (int bb = 0; bb < W; ++bb) {
          int q = q0[i] + bb;
          if (q >= ngy) q -= ngy;
          double *row = grid + 2 * (int64_t)q * ngx;
          const double fv = kv[bb];
          for (int a = 0; a < W; ++a) {
            int p = p0[i] + a;
            if (p >= ngx) p -= ngx;
            const double f = ((p + q) & 1) ? -fv * ku[a] : fv * ku[a];
            row[2 * p] += f * cr;
            row[2 * p + 1] += f * ci;
          }
        }
      }
    }
  }
}

/* Degrid one plane k: out[i] += sum kernel * grid for the listed items. */
void og_degrid_plane(int ngx, int ngy, int W, double beta, int do_w, int k, const int32_t *p0,
                     const int32_t *q0, const int32_t *k0, const double *du, const double *dv,
                     const double *dwf, const int64_t *order, int64_t n, const double *grid,
                     double *out /* re,im per item */, int nthreads) {
  const double scale = 2.0 / W;
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nthreads)
  for (int64_t t = 0; t < n; ++t) {
    const int64_t i = order[t];
    const int aw = k - k0[i];
    if (aw < 0 || aw >= (do_w ? W : 1)) continue;
    double ku[32], kv[32];
    for (int a = 0; a < W; ++a) {
      ku[a] = es((a - du[i]) * scale, beta);
      kv[a] = es((a - dv[i]) * scale, beta);
    }
    double sr = 0.0, si = 0.0;
    for (int bb = 0; bb < W; ++bb) {
      int q = q0[i] + bb;
      if (q >= ngy) q -= ngy;
      const double *row = grid + 2 * (int64_t)q * ngx;
      double rr = 0.0, ri = 0.0;
      for (int a = 0; a < W; ++a) {
        int p = p0[i] + a;
        if (p >= ngx) p -= ngx;
        const double f = ((p + q) & 1) ? -ku[a] : ku[a];
        rr += f * row[2 * p];
        ri += f * row[2 * p + 1];
      }
      sr += kv[bb] * rr;
      si += kv[bb] * ri;
    }
    const double fw = do_w ? es((aw - dwf[i]) * scale, beta) : 1.0;
    out[2 * i] += fw * sr;
    out[2 * i + 1] += fw * si;
  }
}

/* acc[iy*nx+ix] += Re(grid_central(ix, iy) * exp(-2 pi i wk tprime)) */
void og_screen_acc(int nx, int ny, int ngx, int ngy, int do_w, double wk,
                   const double *tprime /* [ny][nx] or NULL */, const double *grid, double *acc,
                   int nthreads) {
  const int ox = (ngx - nx) / 2, oy = (ngy - ny) / 2;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int iy = 0; iy < ny; ++iy) {
    const double *row = grid + 2 * ((int64_t)(iy + oy) * ngx + ox);
    double *a = acc + (int64_t)iy * nx;
    if (!do_w) {
      for (int ix = 0; ix < nx; ++ix) a[ix] += row[2 * ix];
      continue;
    }
    const double *tp = tprime + (int64_t)iy * nx;
    for (int ix = 0; ix < nx; ++ix) {
      double turns = wk * tp[ix];
      turns -= rint(turns);
      const double th = 2.0 * M_PI * turns;
      a[ix] += row[2 * ix] * cos(th) + row[2 * ix + 1] * sin(th);
    }
  }
}

/* grid = 0 outside the central block; image * exp(+2 pi i wk tprime) inside */
void og_screen_pad(int nx, int ny, int ngx, int ngy, int do_w, double wk,
                   const double *tprime, const double *img /* [ny][nx], corrected */,
                   double *grid, int nthreads) {
  const int ox = (ngx - nx) / 2, oy = (ngy - ny) / 2;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int my = 0; my < ngy; ++my) {
    double *row = grid + 2 * (int64_t)my * ngx;
    memset(row, 0, sizeof(double) * 2 * (size_t)ngx);
    const int iy = my - oy;
    if (iy < 0 || iy >= ny) continue;
    const double *im = img + (int64_t)iy * nx;
    double *r = row + 2 * ox;
    if (!do_w) {
      for (int ix = 0; ix < nx; ++ix) r[2 * ix] = im[ix];
      continue;
    }
    const double *tp = tprime + (int64_t)iy * nx;
    for (int ix = 0; ix < nx; ++ix) {
      double turns = wk * tp[ix];
      turns -= rint(turns);
      const double th = 2.0 * M_PI * turns;
      r[2 * ix] = im[ix] * cos(th);
      r[2 * ix + 1] = im[ix] * sin(th);
    }
  }
}

int og_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
