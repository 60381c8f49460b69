"""GPU w-stacking gridder with ducc0.wgridder's interface.

Two levels:

* :class:`Plan` -- sort once, call many times.  Device buffers are torch
  CUDA tensors (torch owns the memory, including the plan's workspace);
  work runs on torch's current CUDA stream.
* :func:`ms2dirty` / :func:`dirty2ms` -- the same arguments, meaning and
  return values as ``ducc0.wgridder.ms2dirty`` / ``dirty2ms`` as RASCIL
  calls them (``rascil/processing_components/imaging/ng.py:91-103,
  232-248``).  The precision follows ducc0's rule: complex128 data run the
  FP64 form, complex64 the FP32 form.
"""

import ctypes

import numpy
import torch

from . import _lib, tuning

_PREC = {"fp32": _lib.GB_FP32, "fp64": _lib.GB_FP64}
_LAYOUT = {"xy": _lib.GB_LAYOUT_XY, "yx": _lib.GB_LAYOUT_YX}
_FFT_MODE = {"auto": 0, "cufft2d": 1, "columns": 2}
FFT_MODE_NAMES = {1: "cufft2d", 2: "columns"}


def _require_cuda(t, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _polmat_arg(polmat):
    if polmat is None:
        return None, None
    m = numpy.ascontiguousarray(numpy.asarray(polmat, dtype=numpy.complex128))
    flat = numpy.ascontiguousarray(m.view(numpy.float64).ravel())
    return flat.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), flat


class Plan:
    """A bound gridding plan for fixed uvw, frequencies and image geometry.

    :param uvw: [nrows, 3] float64 CUDA tensor (metres, u/w as ng.py flips them)
    :param freq: [nchan] float64 CUDA tensor (Hz)
    :param npol: image polarisations gridded together (1, 2, 4)
    :param precision: "fp32" (complex64 data) or "fp64" (complex128 data)
    :param bind: allocate a workspace (torch) and run the bucket sort now; with
        ``bind=False`` call :meth:`bind` with a caller-owned buffer later
    :param fft_mode: "auto" (the library's column kernels where they apply:
        FP32 form, power-of-two grid height), "columns" (require them) or
        "cufft2d" (batched 2-D cuFFT plans); ``info["fft_mode"]`` reports
        the one in use (2 = columns, 1 = cufft2d)
    :param sigma: grid oversampling (1.25, 1.5, 1.75, 2); 0 = the planner's
        choice by its cost model (or a cached autotuning result)
    :param planes_per_batch: w-planes per transform batch (0: what
        ``grid_budget_bytes`` holds)
    :param phase_shift: (s0, s1, s2) of a tangent-plane phase rotation fused
        into the plan's per-item factors: ms2dirty grids vis times
        exp(+2 pi i (u s0 + v s1 + w s2) f/c) (not for a PSF), dirty2ms
        returns predictions times exp(-2 pi i ...); uvw as given to the plan
    """

    def __init__(self, uvw, freq, npix_x, npix_y, pixsize_x, pixsize_y, epsilon,
                 do_wstacking, npol=1, precision="fp32", sigma=0.0, support=0, tile=0,
                 slab=0, grid_budget_bytes=0, bind=True, fft_mode="auto",
                 phase_shift=(0.0, 0.0, 0.0), planes_per_batch=0):
        lib = _lib.load()
        _require_cuda(uvw, "uvw")
        _require_cuda(freq, "freq")
        if uvw.dtype != torch.float64 or freq.dtype != torch.float64:
            raise TypeError("uvw and freq must be float64")
        if uvw.dim() != 2 or uvw.shape[1] != 3:
            raise ValueError("uvw must be [nrows, 3]")
        if precision not in _PREC:
            raise ValueError("precision must be 'fp32' or 'fp64'")
        if fft_mode not in _FFT_MODE:
            raise ValueError("fft_mode must be one of %s" % sorted(_FFT_MODE))
        self.device = uvw.device
        self.precision = precision
        self.npol = int(npol)
        self.nrows, self.nchan = int(uvw.shape[0]), int(freq.shape[0])
        self.npix_x, self.npix_y = int(npix_x), int(npix_y)
        self.shape_key = tuning.shape_key(npix_x, npix_y, pixsize_x, npol, precision, epsilon,
                                          do_wstacking, self.nrows, self.nchan)
        if not sigma and not tile and not slab and not planes_per_batch:
            chosen = tuning.choose(self.shape_key, npix_x, npix_y, self.nrows, self.nchan)
            sigma, tile, slab = chosen["sigma"], chosen["tile"], chosen["slab"]
            planes_per_batch = chosen.get("planes", 0)
            if planes_per_batch:
                grid_budget_bytes = 0
        self._uvw, self._freq = uvw, freq
        p = _lib.PlanParams()
        p.nrows = self.nrows
        p.nchan = self.nchan
        p.npol = self.npol
        p.npix_x = self.npix_x
        p.npix_y = self.npix_y
        p.pixsize_x = float(pixsize_x)
        p.pixsize_y = float(pixsize_y)
        p.epsilon = float(epsilon)
        p.do_wstacking = 1 if do_wstacking else 0
        p.precision = _PREC[precision]
        p.sigma = float(sigma)
        p.support = int(support)
        p.tile = int(tile)
        p.slab = int(slab)
        p.grid_budget_bytes = int(grid_budget_bytes)
        p.fft_mode = _FFT_MODE[fft_mode]
        p.planes_per_batch = int(planes_per_batch)
        shift = [float(x) for x in phase_shift]
        if len(shift) != 3:
            raise ValueError("phase_shift must hold three coefficients")
        p.phase_shift[:] = shift
        self.phase_shift = tuple(shift)
        self._params = p
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(lib.gb_plan_create(ctypes.byref(p), _ptr(uvw), _ptr(freq),
                                          _stream(self.device), ctypes.byref(handle)),
                       "gb_plan_create")
            self._handle = handle
            size = ctypes.c_size_t()
            _lib.check(lib.gb_plan_workspace_size(handle, ctypes.byref(size)))
            self.workspace_bytes = int(size.value)
            self.workspace = None
            if bind:
                self.bind(torch.empty(max(self.workspace_bytes, 256), dtype=torch.uint8,
                                      device=self.device))
        self.info = self._info()

    def bind(self, workspace):
        """Bind device scratch (a uint8 CUDA tensor of at least
        ``workspace_bytes``) and run the bucket sort, on the current stream.
        A plan can be re-bound to another (or the same) buffer at any time;
        the buffer must stay alive while work that uses it runs."""
        _require_cuda(workspace, "workspace")
        if workspace.numel() < self.workspace_bytes:
            raise ValueError("workspace holds %d bytes, the plan needs %d"
                             % (workspace.numel(), self.workspace_bytes))
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().gb_plan_bind(self._handle, _ptr(workspace),
                                                workspace.numel(), _stream(self.device)),
                       "gb_plan_bind")
        self.workspace = workspace

    def _info(self):
        info = _lib.PlanInfo()
        _lib.check(_lib.load().gb_plan_info_get(self._handle, ctypes.byref(info)))
        return info.as_dict()

    @property
    def real_dtype(self):
        return torch.float64 if self.precision == "fp64" else torch.float32

    @property
    def complex_dtype(self):
        return torch.complex128 if self.precision == "fp64" else torch.complex64

    def ms2dirty(self, vis=None, wgt=None, flags=None, polmat=None, psf=False,
                 layout="xy", out=None, sumwt=False):
        """Dirty images [npol, ...] from vis [nrows, nchan, npol_vis].

        :param flags: uint8 or int64 tensor like vis (nonzero = flagged)
        :param polmat: [npol, npol_vis] complex vis-frame -> image-frame matrix
        :param psf: grid (1, 0, ...) per item instead of the data
        :param layout: "xy" (ducc0 dirty[x][y]) or "yx" (RASCIL pixels[y][x])
        :return: dirty tensor (and the per-pol weight sums if sumwt)
        """
        lib = _lib.load()
        if vis is None and not psf:
            raise ValueError("vis is required unless psf=True")
        npv = int(vis.shape[-1]) if vis is not None else (
            int(wgt.shape[-1]) if wgt is not None else self.npol)
        if vis is not None:
            _require_cuda(vis, "vis")
            if vis.dtype != self.complex_dtype:
                raise TypeError("vis must be %s" % self.complex_dtype)
            if vis.numel() != self.nrows * self.nchan * npv:
                raise ValueError("vis must hold nrows * nchan * npol_vis values")
        if wgt is not None:
            _require_cuda(wgt, "wgt")
            if wgt.dtype != self.real_dtype:
                raise TypeError("wgt must be %s" % self.real_dtype)
            if wgt.numel() != self.nrows * self.nchan * npv:
                raise ValueError("wgt must match vis")
        ftype = _lib.GB_FLAGS_NONE
        if flags is not None:
            _require_cuda(flags, "flags")
            if flags.numel() != self.nrows * self.nchan * npv:
                raise ValueError("flags must match vis")
            if flags.dtype == torch.uint8 or flags.dtype == torch.bool:
                ftype = _lib.GB_FLAGS_U8
            elif flags.dtype == torch.int64:
                ftype = _lib.GB_FLAGS_I64
            else:
                raise TypeError("flags must be uint8/bool or int64")
        shape = (self.npol, self.npix_x, self.npix_y) if layout == "xy" else (
            self.npol, self.npix_y, self.npix_x)
        if out is None:
            out = torch.empty(shape, dtype=self.real_dtype, device=self.device)
        else:
            _require_cuda(out, "out")
            if out.dtype != self.real_dtype or out.numel() != shape[0] * shape[1] * shape[2]:
                raise ValueError("out has the wrong dtype or size")
        sw = torch.empty(self.npol, dtype=torch.float64, device=self.device) if sumwt else None
        pm_ptr, _keep = _polmat_arg(polmat)
        with torch.cuda.device(self.device):
            _lib.check(lib.gb_plan_ms2dirty(self._handle, _ptr(vis), npv, _ptr(wgt),
                                            _ptr(flags), ftype, pm_ptr, 1 if psf else 0,
                                            _ptr(out), _LAYOUT[layout], _ptr(sw),
                                            _stream(self.device)), "gb_plan_ms2dirty")
        return (out, sw) if sumwt else out

    def dirty2ms(self, dirty, wgt=None, polmat=None, npol_vis=None, layout="xy", out=None):
        """Visibilities [nrows, nchan, npol_vis] from dirty [npol, ...]."""
        lib = _lib.load()
        _require_cuda(dirty, "dirty")
        if dirty.dtype != self.real_dtype:
            raise TypeError("dirty must be %s" % self.real_dtype)
        if dirty.numel() != self.npol * self.npix_x * self.npix_y:
            raise ValueError("dirty must hold npol images of the plan's size")
        npv = int(npol_vis) if npol_vis else self.npol
        if wgt is not None:
            _require_cuda(wgt, "wgt")
            if wgt.dtype != self.real_dtype or wgt.numel() != self.nrows * self.nchan * npv:
                raise ValueError("wgt has the wrong dtype or size")
        if out is None:
            out = torch.empty((self.nrows, self.nchan, npv), dtype=self.complex_dtype,
                              device=self.device)
        else:
            _require_cuda(out, "out")
            if out.dtype != self.complex_dtype or out.numel() != self.nrows * self.nchan * npv:
                raise ValueError("out has the wrong dtype or size")
        pm_ptr, _keep = _polmat_arg(polmat)
        with torch.cuda.device(self.device):
            _lib.check(lib.gb_plan_dirty2ms(self._handle, _ptr(dirty), _LAYOUT[layout],
                                            _ptr(wgt), pm_ptr, npv, _ptr(out),
                                            _stream(self.device)), "gb_plan_dirty2ms")
        return out

    def device_status(self):
        """Error bits the plan's kernels recorded since the last call (0 =
        none; 1 = a TMA completion wait hit its limit, so that call's output
        is invalid), then cleared.  Waits for the current stream."""
        v = ctypes.c_int32()
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().gb_plan_device_status(self._handle, _stream(self.device),
                                                         ctypes.byref(v)),
                       "gb_plan_device_status")
        return int(v.value)

    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            _lib.load().gb_plan_destroy(self._handle)
            self._handle = None
            self.workspace = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def plan_geometry(npix_x, npix_y, pixsize_x, pixsize_y, epsilon, do_wstacking, w_lo, w_hi,
                  nrows=1, nchan=1, npol=1, precision="fp64", sigma=0.0, support=0):
    """Host-only planner output for a w range (no GPU needed)."""
    p = _lib.PlanParams()
    p.nrows, p.nchan, p.npol = nrows, nchan, npol
    p.npix_x, p.npix_y = npix_x, npix_y
    p.pixsize_x, p.pixsize_y = pixsize_x, pixsize_y
    p.epsilon = epsilon
    p.do_wstacking = 1 if do_wstacking else 0
    p.precision = _PREC[precision]
    p.sigma = sigma
    p.support = support
    info = _lib.PlanInfo()
    _lib.check(_lib.load().gb_plan_geometry(ctypes.byref(p), w_lo, w_hi, ctypes.byref(info)),
               "gb_plan_geometry")
    return info.as_dict()


def _to_device(x, dtype, device):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.from_numpy(numpy.ascontiguousarray(x)).to(device=device, dtype=dtype)


def _precision_of(data, precision):
    if precision is not None:
        return precision
    dt = data.dtype
    if dt in (torch.complex64, torch.float32, numpy.complex64, numpy.float32):
        return "fp32"
    return "fp64"


def ms2dirty(uvw, freq, ms, wgt, npix_x, npix_y, pixsize_x, pixsize_y, nu=0, nv=0,
             epsilon=1e-5, do_wstacking=False, nthreads=1, verbosity=0, mask=None,
             double_precision_accumulation=False, precision=None, device="cuda"):
    """``ducc0.wgridder.ms2dirty`` on the GPU.  ``nu``, ``nv``, ``nthreads``,
    ``verbosity`` and ``double_precision_accumulation`` are accepted and
    ignored (grid accumulation is in the data's precision).  Returns a
    numpy array for numpy input, a CUDA tensor for tensor input."""
    host = not isinstance(ms, torch.Tensor)
    prec = _precision_of(ms, precision)
    rdt = torch.float64 if prec == "fp64" else torch.float32
    cdt = torch.complex128 if prec == "fp64" else torch.complex64
    u = _to_device(uvw, torch.float64, device)
    f = _to_device(numpy.atleast_1d(freq) if not isinstance(freq, torch.Tensor) else freq,
                   torch.float64, device)
    m = _to_device(ms, cdt, device)
    w = _to_device(wgt, rdt, device) if wgt is not None else None
    flags = None
    if mask is not None:
        flags = (_to_device(mask, torch.uint8, device) == 0).to(torch.uint8)
    plan = Plan(u, f, npix_x, npix_y, pixsize_x, pixsize_y, epsilon, do_wstacking, npol=1,
                precision=prec)
    try:
        dirty = plan.ms2dirty(m.reshape(plan.nrows, plan.nchan, 1),
                              None if w is None else w.reshape(plan.nrows, plan.nchan, 1),
                              flags=None if flags is None else flags.reshape(plan.nrows,
                                                                             plan.nchan, 1),
                              layout="xy")[0]
        if host:
            return dirty.cpu().numpy()
        return dirty
    finally:
        plan.close()


def dirty2ms(uvw, freq, dirty, wgt, pixsize_x, pixsize_y, nu=0, nv=0, epsilon=1e-5,
             do_wstacking=False, nthreads=1, verbosity=0, mask=None, precision=None,
             device="cuda"):
    """``ducc0.wgridder.dirty2ms`` on the GPU (see :func:`ms2dirty`)."""
    host = not isinstance(dirty, torch.Tensor)
    prec = _precision_of(dirty, precision)
    rdt = torch.float64 if prec == "fp64" else torch.float32
    u = _to_device(uvw, torch.float64, device)
    f = _to_device(numpy.atleast_1d(freq) if not isinstance(freq, torch.Tensor) else freq,
                   torch.float64, device)
    d = _to_device(dirty, rdt, device)
    npix_x, npix_y = int(d.shape[0]), int(d.shape[1])
    plan = Plan(u, f, npix_x, npix_y, pixsize_x, pixsize_y, epsilon, do_wstacking, npol=1,
                precision=prec)
    try:
        w = None
        if wgt is not None:
            w = _to_device(wgt, rdt, device).reshape(plan.nrows, plan.nchan, 1)
        vis = plan.dirty2ms(d.reshape(1, npix_x, npix_y), wgt=w, layout="xy")
        vis = vis.reshape(plan.nrows, plan.nchan)
        if mask is not None:
            vis = vis * (_to_device(mask, torch.uint8, device) != 0)
        if host:
            return vis.cpu().numpy()
        return vis
    finally:
        plan.close()
