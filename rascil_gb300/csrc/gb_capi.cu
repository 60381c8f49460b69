// C-ABI entry points for invert / predict on a bound plan, and the
// one-shot ducc0-shaped calls.
#include <cmath>
#include <cstring>

#include "gb_plan.cuh"

using namespace gb;

namespace gb {
int make_polmat(const double *host, int nout, int nin, PolMat &pm) {
  memset(&pm, 0, sizeof(pm));
  pm.nout = nout;
  pm.nin = nin;
  if (!host) {
    if (nout != nin) {
      set_error("identity polarisation matrix needs equal pol counts (%d vs %d)", nout, nin);
      return GB_ERR_INVALID_ARG;
    }
    pm.identity = 1;
    return GB_OK;
  }
  for (int i = 0; i < nout * nin; ++i) {
    pm.re[i] = host[2 * i];
    pm.im[i] = host[2 * i + 1];
    pm.fre[i] = (float)pm.re[i];
    pm.fim[i] = (float)pm.im[i];
    if (!std::isfinite(pm.re[i]) || !std::isfinite(pm.im[i])) {
      set_error("polarisation matrix holds a non-finite entry");
      return GB_ERR_INVALID_ARG;
    }
  }
  return GB_OK;
}
}  // namespace gb

extern "C" {

int gb_plan_ms2dirty(gb_plan *p, const void *vis, int32_t npol_vis, const void *wgt,
                     const void *flags, int32_t flags_type, const double *polmat, int32_t psf,
                     void *dirty, int32_t layout, double *sumwt, void *stream) {
  if (!p) {
    set_error("gb_plan_ms2dirty: NULL plan");
    return GB_ERR_INVALID_ARG;
  }
  if (!p->bound) {
    set_error("gb_plan_ms2dirty: plan has no workspace (call gb_plan_bind)");
    return GB_ERR_NOT_BOUND;
  }
  if ((!vis && !psf) || !dirty) {
    set_error("gb_plan_ms2dirty: NULL vis or dirty");
    return GB_ERR_INVALID_ARG;
  }
  if (npol_vis < 1 || npol_vis > 4 || npol_vis < p->g.NP) {
    set_error("npol_vis %d must be in [npol=%d, 4]", npol_vis, p->g.NP);
    return GB_ERR_INVALID_ARG;
  }
  if (flags && flags_type != GB_FLAGS_U8 && flags_type != GB_FLAGS_I64) {
    set_error("flags_type %d unknown", flags_type);
    return GB_ERR_INVALID_ARG;
  }
  if (!flags) flags_type = GB_FLAGS_NONE;
  if (layout != GB_LAYOUT_XY && layout != GB_LAYOUT_YX) {
    set_error("layout %d unknown", layout);
    return GB_ERR_INVALID_ARG;
  }
  PolMat pm;
  int rc = make_polmat(polmat, p->g.NP, npol_vis, pm);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  p->last_stream = s;
  return run_ms2dirty(p, vis, npol_vis, wgt, flags, flags_type, pm, psf, dirty, layout, sumwt, s);
}

int gb_plan_dirty2ms(gb_plan *p, const void *dirty, int32_t layout, const void *wgt,
                     const double *polmat, int32_t npol_vis, void *vis, void *stream) {
  if (!p) {
    set_error("gb_plan_dirty2ms: NULL plan");
    return GB_ERR_INVALID_ARG;
  }
  if (!p->bound) {
    set_error("gb_plan_dirty2ms: plan has no workspace (call gb_plan_bind)");
    return GB_ERR_NOT_BOUND;
  }
  if (!dirty || !vis) {
    set_error("gb_plan_dirty2ms: NULL dirty or vis");
    return GB_ERR_INVALID_ARG;
  }
  if (npol_vis < 1 || npol_vis > 4) {
    set_error("npol_vis %d must be in [1, 4]", npol_vis);
    return GB_ERR_INVALID_ARG;
  }
  if (layout != GB_LAYOUT_XY && layout != GB_LAYOUT_YX) {
    set_error("layout %d unknown", layout);
    return GB_ERR_INVALID_ARG;
  }
  PolMat pm;
  int rc = make_polmat(polmat, npol_vis, p->g.NP, pm);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  p->last_stream = s;
  return run_dirty2ms(p, dirty, layout, wgt, pm, npol_vis, vis, s);
}

static int oneshot(bool invert, const double *uvw, const double *freq, int64_t nrows,
                   int32_t nchan, const void *data_in, const void *wgt, int32_t npix_x,
                   int32_t npix_y, double pixsize_x, double pixsize_y, double epsilon,
                   int32_t do_wstacking, int32_t precision, void *data_out, void *stream) {
  gb_plan_params prm;
  memset(&prm, 0, sizeof(prm));
  prm.nrows = nrows;
  prm.nchan = nchan;
  prm.npol = 1;
  prm.npix_x = npix_x;
  prm.npix_y = npix_y;
  prm.pixsize_x = pixsize_x;
  prm.pixsize_y = pixsize_y;
  prm.epsilon = epsilon;
  prm.do_wstacking = do_wstacking;
  prm.precision = precision;
  gb_plan *p = nullptr;
  int rc = gb_plan_create(&prm, uvw, freq, stream, &p);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  void *ws = nullptr;
  cudaError_t e = cudaMallocAsync(&ws, p->ws_bytes, s);
  if (e != cudaSuccess) {
    gb_plan_destroy(p);
    return cuda_fail(e, "cudaMallocAsync(workspace)");
  }
  rc = gb_plan_bind(p, ws, p->ws_bytes, stream);
  if (!rc) {
    if (invert)
      rc = gb_plan_ms2dirty(p, data_in, 1, wgt, nullptr, GB_FLAGS_NONE, nullptr, 0, data_out,
                            GB_LAYOUT_XY, nullptr, stream);
    else
      rc = gb_plan_dirty2ms(p, data_in, GB_LAYOUT_XY, wgt, nullptr, 1, data_out, stream);
  }
  cudaFreeAsync(ws, s);
  const cudaError_t se = cudaStreamSynchronize(s);
  gb_plan_destroy(p);
  if (rc) return rc;
  if (se != cudaSuccess) return cuda_fail(se, "one-shot call");
  return GB_OK;
}

int gb_ms2dirty(const double *uvw, const double *freq, int64_t nrows, int32_t nchan,
                const void *ms, const void *wgt, int32_t npix_x, int32_t npix_y,
                double pixsize_x, double pixsize_y, double epsilon, int32_t do_wstacking,
                int32_t precision, void *dirty, void *stream) {
  if (!ms || !dirty) {
    set_error("gb_ms2dirty: NULL ms or dirty");
    return GB_ERR_INVALID_ARG;
  }
  return oneshot(true, uvw, freq, nrows, nchan, ms, wgt, npix_x, npix_y, pixsize_x, pixsize_y,
                 epsilon, do_wstacking, precision, dirty, stream);
}

int gb_dirty2ms(const double *uvw, const double *freq, int64_t nrows, int32_t nchan,
                const void *dirty, const void *wgt, int32_t npix_x, int32_t npix_y,
                double pixsize_x, double pixsize_y, double epsilon, int32_t do_wstacking,
                int32_t precision, void *ms, void *stream) {
  if (!dirty || !ms) {
    set_error("gb_dirty2ms: NULL dirty or ms");
    return GB_ERR_INVALID_ARG;
  }
  return oneshot(false, uvw, freq, nrows, nchan, dirty, wgt, npix_x, npix_y, pixsize_x,
                 pixsize_y, epsilon, do_wstacking, precision, ms, stream);
}

}  // extern "C"
