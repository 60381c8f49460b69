/*
 * rascil_gb300 -- C-ABI of the GB300 (sm_103a) w-stacking gridder/degridder.
 *
 * This is the drop-in replacement for the two ducc0 calls that RASCIL's
 * ng imaging path makes:
 *
 *   ducc0.wgridder.ms2dirty  rascil/processing_components/imaging/ng.py:232-248, 259-275
 *   ducc0.wgridder.dirty2ms  rascil/processing_components/imaging/ng.py:91-103, 108-120
 *
 * with the same operator (ducc0 0.24.0 semantics: flipped u/w as ng.py
 * passes them, image axis order [x][y], pixel centre at n/2, 1/n factor
 * when w-stacking).  Work is split into a plan (uvw-dependent: w range,
 * bucket sort of visibilities into uv tiles) and calls that reuse it, so
 * that several polarisations, invert + predict, and repeated autograd
 * calls share one sort.
 *
 * Conventions
 *  - every pointer named *_dev is a device pointer; host pointers say so;
 *  - every call is asynchronous on the caller's CUDA stream (cudaStream_t
 *    passed as void*), except gb_plan_create, which synchronises the
 *    stream once to read the w range back;
 *  - the library never frees caller memory; scratch memory comes from a
 *    caller-provided workspace (gb_plan_workspace_size / gb_plan_bind);
 *  - every entry point returns a gb_status; gb_last_error_string() gives a
 *    message for the calling thread's last failure.  No C++ exception
 *    crosses this boundary.
 */
#ifndef RASCIL_GB300_H
#define RASCIL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  ng.py asserts (ng.py:46,71,158) and wg.py raises
 * ValueError (wg.py:52-54,79-85); here invalid arguments come back as
 * GB_ERR_INVALID_ARG and the Python layer raises ValueError. */
typedef enum {
  GB_OK = 0,
  GB_ERR_INVALID_ARG = 1,
  GB_ERR_NOT_BOUND = 2,
  GB_ERR_WORKSPACE = 3,
  GB_ERR_CUDA = 4,
  GB_ERR_CUFFT = 5,
  GB_ERR_TIMEOUT = 6,
  GB_ERR_INTERNAL = 7,
  GB_ERR_OUT_OF_GRID = 8
} gb_status;

typedef enum { GB_FP32 = 0, GB_FP64 = 1 } gb_precision;

/* How the per-plane 2-D transforms run.  GB_FFT_AUTO picks
 * GB_FFT_COLUMNS where it applies (FP32 form, grid height a power of two
 * from 256 to 32768, twice the image height, even column offset), else
 * GB_FFT_CUFFT_2D.  GB_FFT_COLUMNS: the library's own column kernels,
 * pruned to the image's columns and fused with the w-screen, with its own
 * row kernels for grid widths 4096, 8192 and 16384 (else batched 1-D cuFFT
 * rows); asking for it where it does not apply is GB_ERR_INVALID_ARG.
 * GB_FFT_CUFFT_2D: batched 2-D cuFFT plans plus separate screen passes. */
typedef enum { GB_FFT_AUTO = 0, GB_FFT_CUFFT_2D = 1, GB_FFT_COLUMNS = 2 } gb_fft_mode;

/* Image memory layout.  GB_LAYOUT_XY is ducc0's dirty[x][y] (what
 * ms2dirty returns and dirty2ms takes).  GB_LAYOUT_YX is RASCIL's
 * pixels[..., y, x] (ng.py passes model.T to ducc0, ng.py:94,249), so the
 * Python layer needs no transposes. */
typedef enum { GB_LAYOUT_XY = 0, GB_LAYOUT_YX = 1 } gb_layout;

/* Element type of the optional flags array (nonzero = flagged).  RASCIL's
 * BlockVisibility flags are int64 (memory_data_models.py:1502-1523). */
typedef enum { GB_FLAGS_NONE = 0, GB_FLAGS_U8 = 1, GB_FLAGS_I64 = 2 } gb_flags_type;

typedef struct {
  int64_t nrows;       /* R: uvw rows (times x baselines)                      */
  int32_t nchan;       /* C: frequency channels gridded by this plan           */
  int32_t npol;        /* P: image polarisations gridded together (1, 2, 4)    */
  int32_t npix_x;      /* image size along x (ducc0 npix_x), even, >= 16      */
  int32_t npix_y;      /* image size along y (ducc0 npix_y), even, >= 16      */
  double pixsize_x;    /* radians                                              */
  double pixsize_y;    /* radians                                              */
  double epsilon;      /* requested accuracy (ducc0 epsilon)                   */
  int32_t do_wstacking;/* ducc0 do_wstacking                                   */
  int32_t precision;   /* gb_precision                                         */
  double sigma;        /* grid oversampling (1.25, 1.5, 1.75, 2); 0 = the one of
                          least modelled cost (gridding work against per-plane
                          transform work), 2 unless another is 10 % cheaper */
  int32_t support;     /* kernel support W; 0 = smallest W meeting epsilon     */
  int32_t tile;        /* uv tile side in cells; 0 = default                   */
  int32_t slab;        /* w-planes per bucket slab; 0 = default                */
  int64_t grid_budget_bytes; /* memory for one batch of w-planes; 0 = default  */
  int32_t fft_mode;    /* gb_fft_mode                                          */
  /* Tangent-plane phase rotation fused into the plan (RASCIL's
   * shift_vis_to_image -> phaserotate_visibility, imaging/base.py:67-106,
   * visibility/base.py:296-357,1248-1264).  s = phase_shift in the plan's
   * own uvw frame: ms2dirty grids vis * exp(+2 pi i (u s0 + v s1 + w s2)
   * f/c) (not in PSF mode, whose unit visibilities the reference sets
   * after its rotation); dirty2ms returns its predictions times
   * exp(-2 pi i (u s0 + v s1 + w s2) f/c).  For RASCIL's direction cosines
   * (l, m, n - 1) of the image centre about the visibility phase centre
   * and ng.py's uvw (u and w negated), s = (-l, m, -(n - 1)).  All zero:
   * no rotation.                                                          */
  double phase_shift[3];
  int32_t planes_per_batch; /* w-planes transformed per batch; 0 = as many as
                               grid_budget_bytes holds (at least one)        */
} gb_plan_params;

/* Geometry the planner chose; all host values. */
typedef struct {
  int32_t support, ngrid_x, ngrid_y, nplanes, planes_per_batch, tile, slab;
  double beta, sigma, dw, w_lo, w_hi, tc;
  int64_t nitems, nbuckets, workspace_bytes;
  int32_t fft_mode;    /* the gb_fft_mode in use (never GB_FFT_AUTO)           */
  int32_t own_rows;    /* 1: GB_FFT_COLUMNS with the library's row transforms
                          (grid width 4096, 8192 or 16384: no cuFFT plan, rows
                          without visibilities skipped); 0: cuFFT rows      */
} gb_plan_info;

typedef struct gb_plan gb_plan;

/* Host-only planning: the geometry for a given w range, without a GPU.
 * Mirrors what gb_plan_create computes after its w-range reduction. */
int gb_plan_geometry(const gb_plan_params *params, double w_lo, double w_hi,
                     gb_plan_info *info_out);

/* Create a plan for the visibility coordinates uvw_dev [nrows][3] (metres,
 * float64) at freq_dev [nchan] (Hz, float64).  Reduces the w range on
 * the device and synchronises `stream` once.  Replaces the per-call setup
 * inside ducc0.wgridder.ms2dirty/dirty2ms (ng.py:91-120,232-275). */
int gb_plan_create(const gb_plan_params *params, const double *uvw_dev,
                   const double *freq_dev, void *stream, gb_plan **plan_out);

/* Bytes of device scratch the plan needs (16-byte aligned start). */
int gb_plan_workspace_size(const gb_plan *plan, size_t *bytes_out);

/* Bind scratch memory and run the device-side bucket sort of all
 * (row, channel) items into (w-slab, uv-tile) buckets.  Asynchronous. */
int gb_plan_bind(gb_plan *plan, void *workspace_dev, size_t workspace_bytes,
                 void *stream);

int gb_plan_info_get(const gb_plan *plan, gb_plan_info *info_out);

/* Verification export of the bucket sort: for every item i = row * nchan +
 * chan, its bucket id (slab-major, then v-tile, then u-tile), first support
 * cell (p0, q0, k0) and offsets (du, dv, dwf) as stored.  Any output may
 * be NULL.  No counterpart in the reference (ducc0 keeps its index
 * internal); it lets tests prove the device sort is bit-exact. */
int gb_plan_export_items(const gb_plan *plan, uint32_t *bucket_dev, int32_t *cell_dev,
                         double *frac_dev, void *stream);

/* Release host resources (cuFFT plans).  Never frees the workspace. */
int gb_plan_destroy(gb_plan *plan);

/* Device status of a bound plan: waits for `stream`, returns in *status_out
 * the error bits kernels recorded since the last call (0 = none; 1 = a
 * TMA completion wait ran past its iteration limit, so that call's output
 * is invalid) and clears them.  No counterpart in the reference (its CPU
 * gridder has no device waits). */
int gb_plan_device_status(gb_plan *plan, void *stream, int32_t *status_out);

/* Invert: dirty image from visibilities.  Replaces ducc0 ms2dirty
 * (ng.py:232-248 MFS, 259-275 per channel) for all npol polarisations
 * in one pass.
 *   vis_dev     [nrows][nchan][npol_vis] complex64 (GB_FP32) or complex128
 *   wgt_dev     [nrows][nchan][npol_vis] float32 / float64, or NULL (= 1)
 *   flags_dev   [nrows][nchan][npol_vis] of flags_type, or NULL
 *   polmat_host npol x npol_vis complex (re, im interleaved, float64):
 *               vis-frame -> image-frame matrix, or NULL for identity
 *               (convert_pol_frame, rascil/data_models/polarisation.py:367-419)
 *   psf         nonzero: grid (1, 0, ...) instead of the data (ng.py:223-225)
 *   dirty_dev   [npol] images of float32 / float64 in `layout`
 *   sumwt_dev   [npol] float64 sums of (flagged) weights, or NULL
 */
int gb_plan_ms2dirty(gb_plan *plan, const void *vis_dev, int32_t npol_vis,
                     const void *wgt_dev, const void *flags_dev,
                     int32_t flags_type, const double *polmat_host, int32_t psf,
                     void *dirty_dev, int32_t layout, double *sumwt_dev,
                     void *stream);

/* Predict: visibilities from a model image.  Replaces ducc0 dirty2ms
 * (ng.py:91-103 MFS, 108-120 per channel) for all npol polarisations.
 *   dirty_dev   [npol] real images (float32 / float64) in `layout`
 *   wgt_dev     [nrows][nchan][npol_vis] or NULL (ng.py passes None)
 *   polmat_host npol_vis x npol complex: image-frame -> vis-frame, or NULL
 *   vis_dev     [nrows][nchan][npol_vis] complex64 / complex128 (written)
 */
int gb_plan_dirty2ms(gb_plan *plan, const void *dirty_dev, int32_t layout,
                     const void *wgt_dev, const double *polmat_host,
                     int32_t npol_vis, void *vis_dev, void *stream);

/* One-shot ducc0-shaped calls (single polarisation, [nrows][nchan] data,
 * dirty in [npix_x][npix_y]); allocate scratch with cudaMallocAsync on
 * `stream` and free it before returning.  Same arguments and meaning as
 * ducc0.wgridder.ms2dirty / dirty2ms as called at ng.py:232-248 / 91-103. */
int gb_ms2dirty(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                int32_t nchan, const void *ms_dev, const void *wgt_dev,
                int32_t npix_x, int32_t npix_y, double pixsize_x,
                double pixsize_y, double epsilon, int32_t do_wstacking,
                int32_t precision, void *dirty_dev, void *stream);

int gb_dirty2ms(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                int32_t nchan, const void *dirty_dev, const void *wgt_dev,
                int32_t npix_x, int32_t npix_y, double pixsize_x,
                double pixsize_y, double epsilon, int32_t do_wstacking,
                int32_t precision, void *ms_dev, void *stream);

/* Component DFT: vis_dev[r][c][p] = sum_k flux[k][c][p] *
 * exp(-2 pi i (uvw[r] f_c / c) . lmn[k]), lmn rows (l, m, n-1).  Replaces
 * dft_kernel / dft_gpu_raw_kernel
 * (rascil/processing_components/imaging/dft.py:123-178, 284-332).
 *   lmn_dev   [ncomp][3] float64;  flux_dev [ncomp][nchan][npol] complex128
 *   vis_dev   [nrows][nchan][npol] complex64 (GB_FP32) or complex128 (GB_FP64)
 *   exact     nonzero: FP64 sincos; zero: FP64 phase, FP32 sincos */
int gb_dft_components(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                      int32_t nchan, const double *lmn_dev, const double *flux_dev,
                      int32_t ncomp, int32_t npol, void *vis_dev, int32_t vis_precision,
                      int32_t exact, void *stream);

/* Exact dirty-image values at pixels pix_dev [npix][2] (ix, iy) in ducc0's
 * ms2dirty convention, for polarisation `pol` of ms [nrows][nchan][npol]
 * (complex64 / complex128 per ms_precision) with optional weights of the
 * same real precision.  The direct sum the gridder approximates; used as
 * the oracle at sizes the CPU cannot reach.  No counterpart in the
 * reference (its tests compare against the DFT of components instead). */
int gb_dft_pixels(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                  int32_t nchan, int32_t npol, int32_t pol, const void *ms_dev,
                  int32_t ms_precision, const void *wgt_dev, const int32_t *pix_dev,
                  int32_t npix, int32_t npix_x, int32_t npix_y, double pixsize_x,
                  double pixsize_y, int32_t do_wstacking, int32_t exact, double *out_dev,
                  void *stream);

/* Per-antenna complex gains (differentiable predict).  No counterpart in
 * the reference's ng path; RASCIL applies gains in its calibration code
 * (rascil/processing_components/calibration/operations.py) on the host.
 *   gains_dev   [nant][nchan] complex128;  ant1_dev/ant2_dev [nrows] int32
 *   vis/out     [nrows][nchan][npol] complex64 (GB_FP32) or complex128
 * gb_apply_gains:   out = g[ant1] conj(g[ant2]) vis
 * gb_gain_gradient: grad_gains += d L / d gains for a real loss L whose
 *                   gradient with respect to `out` is grad_dev (dL/dRe + i dL/dIm);
 *                   grad_gains_dev is accumulated, not overwritten. */
int gb_apply_gains(const void *vis_dev, const double *gains_dev, const int32_t *ant1_dev,
                   const int32_t *ant2_dev, int64_t nrows, int32_t nchan, int32_t npol,
                   int32_t precision, void *out_dev, void *stream);
int gb_gain_gradient(const void *vis_dev, const void *grad_dev, const double *gains_dev,
                     const int32_t *ant1_dev, const int32_t *ant2_dev, int64_t nrows,
                     int32_t nchan, int32_t npol, int32_t nant, int32_t precision,
                     double *grad_gains_dev, void *stream);

/* Kernel profiling (process-wide).  While enabled, every launch of this
 * library's kernels and cuFFT executions records a CUDA-event pair on its
 * stream and the algorithmic bytes it must move; gb_profile_get waits for
 * the recorded events and returns per-kernel totals.  No counterpart in
 * the reference (its timing is wall-clock around invert_ng, rascil/
 * processing_components/util/performance.py:40-296). */
int gb_profile_enable(int32_t on);
int gb_profile_reset(void);
int gb_profile_count(void);
int gb_profile_get(int32_t index, char *name, int32_t name_len, double *total_ms,
                   int64_t *launches, double *bytes);
/* Kernel-weighted updates of the gridding / degridding kernels recorded
 * under profiling index `index`: one per (item, polarisation, grid cell of
 * its W x W support, w-plane its support reaches).  0 for other kernels,
 * and while per-plane statistics are unavailable.  No counterpart in the
 * reference. */
int gb_profile_updates(int32_t index, double *updates);

/* Measured shared-memory peaks of the current GPU, for the gridder's and
 * degridder's update-rate rooflines: conflict-free 32-bit integer atomic
 * adds per second and conflict-free 8-byte loads per second over all SMs.
 * Synchronises `stream`.  No counterpart in the reference. */
int gb_probe_smem_peaks(double *atomics_per_s, double *loads8_per_s, void *stream);

/* Allocation-free w range.  For callers that cannot allocate device memory
 * where they need it -- a host framework that owns every device buffer, or
 * a real-time pipeline that forbids allocation after start-up -- this does
 * the w-range reduction gb_plan_create performs (which takes its scratch
 * from cudaMallocAsync) with its scratch in a fixed 384 KiB device array
 * instead, and calls no allocating routine.  No counterpart in the
 * reference.
 *   uvw_dev [nrows][3] metres, freq_dev [nchan] Hz (float64, device)
 *   out_dev [4] float64 (device): w_lo, w_hi, the range of |w| in
 *           wavelengths (a w-stacking plan mirrors rows with w < 0 to -uvw)
 *           over all (row, channel) items with a finite uvw row and a
 *           positive, finite frequency, then the number of rows with a non-finite coordinate
 *           and the number of non-positive or non-finite frequencies.  For
 *           input the planner accepts (both counts zero) and a w-stacking
 *           plan, w_lo and w_hi are bit-identical to gb_plan_info's; plans
 *           without w-stacking report 0, 0 there.  When every row or every
 *           frequency is invalid, w_lo = +inf and w_hi = -inf.
 * At most 67,108,864 rows per call (GB_ERR_INVALID_ARG beyond).  A call
 * outside a stream capture looks up the array's device address on the
 * current device (a context recreated after cudaDeviceReset gets a new
 * one); a call inside a capture reuses the address from the last call on
 * that device outside a capture, so make one call before any capture.  All
 * calls share the array: calls that overlap on the GPU (other streams,
 * other host threads) race, and the caller must serialise them. */
int gb_wrange_noalloc(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                      int32_t nchan, double *out_dev, void *stream);

/* Imaging weights: RASCIL's weight_visibility
 * (rascil/processing_components/imaging/weighting.py:27-48, with
 * grid_blockvisibility_weight_to_griddata and griddata_blockvisibility_reweight,
 * griddata/gridding.py:260-425).  The flagged imaging weights are gridded on
 * the image-sized uv grid (cell of a sample: round((u f/c) / cdelt_u + nx/2)
 * with cdelt_u = 1 / (nx cdelt_x_deg pi/180), likewise v), then every
 * sample's imaging weight becomes
 *   GB_WEIGHT_UNIFORM  w (w / G),
 *   GB_WEIGHT_ROBUST   w (1 + f2 w) / (1 + f2 G), f2 = (5 10^-R)^2 sum(w) / sum(G^2),
 *   (0 where G <= 0), or for GB_WEIGHT_NATURAL the weight itself.
 *   uvw_dev       [nrows][3] f64 metres (as stored, no sign flips)
 *   freq_dev      [nchan] f64 Hz; vis_to_im_dev [nchan] i32 image channel of each
 *   weight_dev, imaging_weight_dev  [nrows][nchan][npol] f64
 *   flags_dev     [nrows][nchan][npol] of flags_type, or NULL (GB_FLAGS_NONE)
 *   cdelt_x_deg, cdelt_y_deg  the image WCS's cdelt[0], cdelt[1] (degrees)
 *   grid_dev      [nchan_img][ny][nx][npol] f64 scratch: on return the gridded weights G
 *                 (natural), else per cell 1 / G (uniform) or 1 / (1 + f2 G) (robust), 0
 *                 where G <= 0
 *   cells_dev     [nrows][nchan] u32 scratch: each sample's cell v * nx + u
 *   imaging_weight_out_dev  [nrows][nchan][npol] f64 (may alias neither input)
 *   sums_dev      [2] f64: sum(G), sum(G^2) on return
 * Synchronises `stream` (to report) and returns GB_ERR_OUT_OF_GRID when a
 * sample's cell lies outside the grid (the reference asserts). */
typedef enum { GB_WEIGHT_NATURAL = 0, GB_WEIGHT_UNIFORM = 1, GB_WEIGHT_ROBUST = 2 } gb_weighting;
int gb_weight_visibility(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                         int32_t nchan, int32_t npol, const int32_t *vis_to_im_dev,
                         int32_t nchan_img, int32_t nx, int32_t ny, double cdelt_x_deg,
                         double cdelt_y_deg, const double *weight_dev,
                         const double *imaging_weight_dev, const void *flags_dev,
                         int32_t flags_type, int32_t weighting, double robustness,
                         double *grid_dev, uint32_t *cells_dev,
                         double *imaging_weight_out_dev, double *sums_dev, void *stream);

/* A list of independent solves (many snapshots of uneven size) issued in
 * one call: plan i is bound to workspace i % nslots and runs on stream
 * i % nslots -- its bucket sort, then ms2dirty of vis[i] into dirty[i] and
 * dirty2ms of model[i] into pred[i] (either may be NULL, arrays included),
 * with unit weights, no flags and the identity pol matrix -- so the slots'
 * work overlaps while each slot's plans run in order on their shared
 * workspace.  Each workspace holds at least the largest workspace_size of
 * its plans.  Asynchronous; capturable in a CUDA graph.  Replaces the
 * reference's per-snapshot Dask tasks over invert/predict
 * (workflows/rsexecute/imaging/imaging_rsexecute.py:72-157) for a list of
 * blocks already on the device. */
int gb_batch_run(gb_plan *const *plans, int32_t nplans, void *const *workspaces,
                 const size_t *workspace_bytes, void *const *streams, int32_t nslots,
                 const void *const *vis, void *const *dirty, const void *const *model,
                 void *const *pred, int32_t layout);

/* The same program with every solve's full argument list: the invert and
 * predict arguments of gb_plan_ms2dirty / gb_plan_dirty2ms per plan, so the
 * list workflows (invert_list / predict_list over blocks with flags,
 * imaging weights and polarisation frames, imaging_rsexecute.py:72-157)
 * run as one device program.  Per round, the gridding of every slot's
 * current plan runs in one persistent launch per (polarisations, lane
 * width) and the degridding in one per (polarisations, support, output
 * polarisation matrix), each fed from a device work queue; bucket sorts,
 * transforms and screens run on the slot streams.  nslots <= 16; streams[0]
 * carries the launches shared by all slots and ends after all the work.
 * Asynchronous; capturable in a CUDA graph. */
typedef struct {
  /* invert (vis or psf non-zero: grid; else skipped) */
  const void *vis;           /* [nrows][nchan][npol_vis] complex, or NULL with psf   */
  int32_t npol_vis;
  int32_t psf;
  const void *wgt;           /* like vis, real; NULL = 1                              */
  const void *flags;         /* like vis, flags_type; NULL = none                     */
  int32_t flags_type;
  int32_t pad0;
  const double *polmat_in;   /* host, npol x npol_vis complex; NULL = identity        */
  void *dirty;               /* [npol] images in `layout`                             */
  double *sumwt;             /* [npol] or NULL                                        */
  /* predict (model non-NULL: degrid; else skipped) */
  const void *model;         /* [npol] images in `layout`                             */
  const double *polmat_out;  /* host, npol_out x npol complex; NULL = identity        */
  int32_t npol_out;
  int32_t pad1;
  void *pred;                /* [nrows][nchan][npol_out] complex (written)            */
} gb_batch_item;
int gb_batch_run_items(gb_plan *const *plans, const gb_batch_item *items, int32_t nplans,
                       void *const *workspaces, const size_t *workspace_bytes,
                       void *const *streams, int32_t nslots, int32_t layout);

/* Tangent-plane phase rotation of visibilities in place, RASCIL's
 * phaserotate_visibility(tangent=True) (visibility/base.py:296-357) with
 * the phasor of calculate_blockvisibility_phasor (:1248-1264):
 *   vis[r][c][p] *= exp(+2 pi i d)   (inverse = 0: times conj(phasor))
 *   vis[r][c][p] *= exp(-2 pi i d)   (inverse = 1: times phasor)
 * with d = (uvw[r] f_c / c) . (s_l, s_m, s_n), formed in FP64; s is
 * (l, m, sqrt(1 - l^2 - m^2) - 1) of the new phase centre about the old.
 *   uvw_dev [nrows][3] f64 metres; freq_dev [nchan] f64 Hz
 *   vis_dev [nrows][nchan][npol] complex64 (GB_FP32) or complex128 (GB_FP64)
 * Asynchronous on `stream`.  invert/predict do not need it: they fuse the
 * rotation through gb_plan_params.phase_shift. */
int gb_phase_rotate(const double *uvw_dev, const double *freq_dev, int64_t nrows,
                    int32_t nchan, int32_t npol, void *vis_dev, int32_t precision, double s_l,
                    double s_m, double s_n, int32_t inverse, void *stream);

/* Message for the calling thread's last non-GB_OK status. */
const char *gb_last_error_string(void);

/* Library version string. */
const char *gb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* RASCIL_GB300_H */
