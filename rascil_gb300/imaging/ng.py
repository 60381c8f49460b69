"""Drop-in ``invert_ng`` / ``predict_ng`` on the GB300 gridder.

Same signatures, keyword arguments, defaults and results as
``rascil/processing_components/imaging/ng.py`` (``predict_ng`` ``:33-133``,
``invert_ng`` ``:136-282``), with the ducc0 calls replaced by one plan per
(set of channels) on the GPU:

* the u and w flips of ``ng.py:73-77,201-204`` are applied on the device;
* all polarisations are gridded in one pass; ``convert_pol_frame`` and
  the flagging (``flagged_vis`` / ``flagged_imaging_weight``) are fused
  into the kernels as a pol matrix and a flags array;
* images are read and written in RASCIL's [pol][y][x] order, so the
  ``.T`` of ``ng.py:94,249`` costs nothing;
* MFS (``ng.py:227-250``): one plan over all channels.  Per-channel
  (``ng.py:251-277``): one plan per image channel over the visibility
  channels that map to it (their sum is what ng.py accumulates);
* ``shift_vis_to_image`` (``ng.py:129-130,169-170``, a tangent-plane phase
  rotation when the image centre is not the visibilities' phase centre) is
  fused into the plan's per-item phase factors, so it costs no pass and no
  copy of the visibilities;
* images accumulate and are normalised by sumwt on the device; host
  arrays in page-locked memory move by direct DMA, and results come back
  into page-locked arrays (torch's host caching allocator).

Extra keyword arguments: ``precision`` ("fp64", the default, matches
the reference's complex128 path; "fp32" is the fast form), ``device``,
``grid_budget_bytes`` (device memory for one batch of w-planes).
``threads`` and ``verbosity`` are accepted and ignored.
"""

import logging
import os
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy
import torch

from ..data_models import copy_visibility
from ..polarisation import conversion_matrix
from ..wgridder import Plan
from .base import fused_phase_shift, image_is_canonical

log = logging.getLogger("rascil-logger")

__all__ = ["predict_ng", "invert_ng", "residual_ng", "predict_gb", "invert_gb", "clear_plan_cache"]


def _budget(kwargs):
    """Device memory for one batch of w-planes (``grid_budget_bytes``, extra
    keyword; 0 = the library default)."""
    return int(get_parameter(kwargs, "grid_budget_bytes", 0))


def get_parameter(kwargs, key, default=None):
    """``rascil/data_models/parameters.py:108-125``: kwargs lookup with default."""
    if kwargs is None:
        return default
    value = kwargs.get(key, default)
    return default if value is None else value


def _vis_to_im(model, freq):
    return numpy.round(model.image_acc.wcs.sub([4]).wcs_world2pix(freq, 0)[0]).astype("int")


def _device_uvw(uvw, device, nan_to_num=False):
    u = _to_device(numpy.ascontiguousarray(uvw.reshape(-1, 3), dtype=numpy.float64), None,
                   device)
    if nan_to_num:
        u = torch.nan_to_num(u)
    u[:, 0].neg_()
    u[:, 2].neg_()
    return u


def _to_device(x, dtype, device):
    """Host array -> device tensor.  From page-locked memory the copy is a
    direct DMA; a dtype conversion (dtype not None) happens on the device."""
    t = torch.from_numpy(numpy.ascontiguousarray(x))
    t = t.to(device=device, non_blocking=t.is_pinned())
    return t if dtype is None else t.to(dtype)


def _torch_dtype(np_dtype):
    return torch.from_numpy(numpy.zeros(0, dtype=np_dtype)).dtype


def _to_host(t, dtype):
    """Device tensor -> numpy array in page-locked memory (torch's host
    caching allocator), so the copy is a direct DMA."""
    host = torch.empty(t.shape, dtype=dtype, pin_memory=t.is_cuda)
    host.copy_(t)
    return host.numpy()


# One-entry plan cache: RASCIL pipelines call invert_ng and predict_ng on the
# same visibilities, so the second call can reuse the first one's plan (its
# bucket sort and tables) instead of building it again.  A cached plan is
# reused only when the geometry and parameters match and the uvw just
# uploaded are equal, element for element on the device, to the plan's own.
# A plan in use is checked out of the cache, so concurrent callers never
# share one.  RASCIL_GB300_PLAN_CACHE=0 disables it.
#
# Callers may run on different CUDA streams (the list workflows run one per
# worker thread): a plan or workspace handed back carries an event recorded
# on its last user's stream, the next user's stream waits on it, and every
# stream that uses a workspace is recorded on the tensor so the caching
# allocator never reuses it under pending work.
_plan_cache = {}
_spare_ws = []  # at most one (workspace, event) of a closed plan, reused by the next
_plan_lock = threading.Lock()


def _cache_on():
    return os.environ.get("RASCIL_GB300_PLAN_CACHE", "1") != "0"


def _mark_used(ws, event=None):
    """The current stream is about to use ``ws``: order it after ``event``
    and keep the allocator from recycling ``ws`` before this stream is done."""
    stream = torch.cuda.current_stream(ws.device)
    if event is not None:
        stream.wait_event(event)
    ws.record_stream(stream)


def _done_event(device):
    ev = torch.cuda.Event()
    ev.record(torch.cuda.current_stream(device))
    return ev


def _retire(plan, event):
    """Close a plan and keep its workspace for the next plan (a multi-GB
    buffer; allocating it anew each call costs more than the transfers)."""
    ws = plan.workspace
    plan.close()
    if ws is None:
        return
    with _plan_lock:
        keep = [w for w in _spare_ws + [(ws, event)] if w[0].device == ws.device]
        keep.sort(key=lambda w: w[0].numel())
        _spare_ws[:] = keep[-1:]


def _new_plan(uvw, f, nx, ny, pixsize, epsilon, do_wstacking, npol, precision, shift,
              budget=0):
    plan = Plan(uvw, f, nx, ny, pixsize, pixsize, epsilon, do_wstacking, npol=npol,
                precision=precision, bind=False, phase_shift=shift, grid_budget_bytes=budget)
    need = max(plan.workspace_bytes, 256)
    spare = None
    with _plan_lock:
        for i, (w, _) in enumerate(_spare_ws):
            if w.device == uvw.device and w.numel() >= need:
                spare = _spare_ws.pop(i)
                break
    if spare is None:
        ws = torch.empty(need, dtype=torch.uint8, device=uvw.device)
    else:
        ws = spare[0]
        _mark_used(ws, spare[1])
    plan.bind(ws)
    return plan


def _checkout_plan(uvw, f, nx, ny, pixsize, epsilon, do_wstacking, npol, precision, shift,
                   budget=0):
    """(key, (uvw, plan)) for the current stream: the cached plan when it
    fits, else a new one."""
    key = (uvw.device, tuple(uvw.shape), tuple(f.cpu().tolist()), nx, ny, float(pixsize),
           float(epsilon), bool(do_wstacking), int(npol), precision, tuple(shift), int(budget))
    if _cache_on():
        with _plan_lock:
            hit = _plan_cache.pop(key, None)
        if hit is not None:
            cached_uvw, plan, event = hit
            torch.cuda.current_stream(uvw.device).wait_event(event)
            if torch.equal(cached_uvw, uvw):
                _mark_used(plan.workspace)
                return key, (cached_uvw, plan)
            _retire(plan, event)
    return key, (uvw, _new_plan(uvw, f, nx, ny, pixsize, epsilon, do_wstacking, npol, precision,
                                shift, budget))


def _checkin_plan(key, entry):
    """Hand a plan back once the current stream has queued all its work."""
    uvw, plan = entry
    event = _done_event(uvw.device)
    if not _cache_on():
        _retire(plan, event)
        return
    with _plan_lock:
        old = list(_plan_cache.values())
        _plan_cache.clear()
        _plan_cache[key] = (uvw, plan, event)
    for _, p, ev in old:
        _retire(p, ev)


def clear_plan_cache(release_memory=False):
    """Drop the cached plan, so the next call sorts its visibilities again.
    Its device workspace is kept for the next plan unless release_memory."""
    with _plan_lock:
        old = list(_plan_cache.values())
        _plan_cache.clear()
    for _, plan, ev in old:
        _retire(plan, ev)
    if release_memory:
        with _plan_lock:
            _spare_ws.clear()


# Host threads for predict_ng's deep copy of its input (see predict_ng).
_copy_pool = []
_copy_pool_lock = threading.Lock()


def _host_pool():
    with _copy_pool_lock:
        if not _copy_pool:
            _copy_pool.append(ThreadPoolExecutor(max_workers=4,
                                                 thread_name_prefix="rascil_gb300_copy"))
        return _copy_pool[0]


def predict_ng(bvis, model, **kwargs):
    """Predict visibilities from a model image (``ng.py:33-133``)."""
    assert image_is_canonical(model)
    if model is None:
        return bvis
    epsilon = get_parameter(kwargs, "epsilon", 1e-12)
    do_wstacking = get_parameter(kwargs, "do_wstacking", True)
    precision = get_parameter(kwargs, "precision", "fp64")
    device = torch.device(get_parameter(kwargs, "device", "cuda"))
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    rdt = torch.float64 if precision == "fp64" else torch.float32

    freq = numpy.asarray(bvis.frequency.data, dtype=numpy.float64)
    nrows, nbaselines, vnchan, vnpol = bvis.vis.shape
    m_nchan, m_npol, ny, nx = model["pixels"].data.shape
    assert m_npol == vnpol
    pixsize = abs(numpy.radians(model.image_acc.wcs.wcs.cdelt[0]))
    vis_to_im = _vis_to_im(model, freq)
    # shift_vis_to_image(..., inverse=True) of ng.py:130, fused into the plan
    rotates, shift = fused_phase_shift(bvis, model)
    polmat = conversion_matrix(model.image_acc.polarisation_frame,
                               bvis.blockvisibility_acc.polarisation_frame)
    pm = None if numpy.array_equal(polmat, numpy.eye(vnpol)) else polmat
    if nrows * nbaselines == 0 or vnchan == 0:
        # no samples to predict: the zeroed copy ng.py:56 starts from
        newbvis = copy_visibility(bvis, zero=True)
        if rotates:
            newbvis.attrs["phasecentre"] = model.image_acc.phasecentre
        return newbvis
    # ng.py:56 deep-copies the input (flags, weights, uvw: several times the
    # visibilities' bytes); the copy runs on a host thread while the GPU
    # predicts, and then takes the predicted visibilities as its vis
    copy_job = _host_pool().submit(copy_visibility, bvis, skip_vis=True)
    uvw = _device_uvw(bvis.uvw.data, device, nan_to_num=True)
    pixels = model["pixels"].data
    out = torch.empty((nrows * nbaselines, vnchan, vnpol), dtype=cdt, device=device)
    if m_nchan == 1:
        groups = [(0, numpy.arange(vnchan))]
    else:
        groups = [(ic, numpy.nonzero(vis_to_im == ic)[0]) for ic in numpy.unique(vis_to_im)]
    for ichan, chans in groups:
        f = torch.from_numpy(numpy.ascontiguousarray(freq[chans])).to(device)
        key, entry = _checkout_plan(uvw, f, nx, ny, pixsize, epsilon, do_wstacking, m_npol,
                                    precision, shift, _budget(kwargs))
        try:
            img = _to_device(pixels[ichan], rdt, device)
            vis = entry[1].dirty2ms(img, polmat=pm, npol_vis=vnpol, layout="yx")
        finally:
            _checkin_plan(key, entry)
        if len(chans) == vnchan:
            out = vis
        else:
            out[:, torch.from_numpy(chans).to(device), :] = vis
    vdt = bvis["vis"].data.dtype
    out = out.reshape(nrows, nbaselines, vnchan, vnpol)
    if vdt == numpy.complex128 and out.dtype != torch.complex128:
        out = out.to(torch.complex128)
    elif vdt == numpy.complex64 and out.dtype != torch.complex64:
        out = out.to(torch.complex64)
    result = _to_host(out, out.dtype)
    if result.dtype != vdt:
        result = result.astype(vdt)
    # the zeroed vis of ng.py:56's copy would be overwritten: the copy gets
    # the predicted visibilities directly instead
    newbvis = copy_job.result()
    newbvis["vis"].data = result
    if rotates:
        newbvis.attrs["phasecentre"] = model.image_acc.phasecentre
    return newbvis


def invert_ng(bvis, model, dopsf=False, normalise=True, **kwargs):
    """Invert visibilities to (image, sumwt) (``ng.py:136-282``)."""
    return _invert(bvis, model, dopsf, normalise, None, kwargs)


def residual_ng(bvis, model, normalise=True, **kwargs):
    """Residual image and sumwt of ``bvis`` against ``model``: what RASCIL's
    residual workflow computes as ``invert_ng(vis - predict_ng(zeroed copy
    of vis, model), model)`` (``imaging_rsexecute.py:160-181``, with
    ``zero_list`` / ``subtract_list`` ``:844-892``), done in one pass on the
    GPU: the visibilities are uploaded once, each channel group's plan is
    shared by the predict and the invert, and the model visibilities and
    their difference never leave the device.  The model is also the image
    template, as in the workflow."""
    if numpy.isnan(numpy.asarray(bvis.uvw.data)).any():
        # predict_ng and invert_ng treat non-finite uvw differently; compose them
        pred = predict_ng(bvis, model, **kwargs)
        return invert_ng(copy_visibility(bvis, vis=bvis["vis"].data - pred["vis"].data), model,
                         normalise=normalise, **kwargs)
    return _invert(bvis, model, False, normalise, model, kwargs)


def _invert(bvis, model, dopsf, normalise, residual_of, kwargs):
    """invert_ng, or with ``residual_of`` (a model image) the invert of
    vis minus that model's prediction."""
    assert image_is_canonical(model)
    im = model
    epsilon = get_parameter(kwargs, "epsilon", 1e-12)
    do_wstacking = get_parameter(kwargs, "do_wstacking", True)
    precision = get_parameter(kwargs, "precision", "fp64")
    device = torch.device(get_parameter(kwargs, "device", "cuda"))
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    rdt = torch.float64 if precision == "fp64" else torch.float32

    # shift_vis_to_image of ng.py:169-170, fused into the plan: the gridder
    # multiplies by the phase factor, so the visibilities are not copied
    _, shift = fused_phase_shift(bvis, im)
    freq = numpy.asarray(bvis.frequency.data, dtype=numpy.float64)
    nrows, nbaselines, vnchan, vnpol = bvis.vis.shape
    nchan, npol, ny, nx = im["pixels"].data.shape
    pixsize = abs(numpy.radians(im.image_acc.wcs.wcs.cdelt[0]))
    polmat = conversion_matrix(bvis.blockvisibility_acc.polarisation_frame,
                               im.image_acc.polarisation_frame)
    pm = None if (npol == vnpol and numpy.array_equal(polmat, numpy.eye(vnpol))) else polmat
    pred_pm = None
    if residual_of is not None:
        assert npol == vnpol
        pmat = conversion_matrix(im.image_acc.polarisation_frame,
                                 bvis.blockvisibility_acc.polarisation_frame)
        pred_pm = None if numpy.array_equal(pmat, numpy.eye(vnpol)) else pmat
    vis_to_im = _vis_to_im(model, freq)
    R = nrows * nbaselines
    if R == 0 or vnchan == 0:
        # no samples: ms2dirty grids nothing, the weight sums stay 0 and
        # normalise_sumwt leaves a zero image (ng.py:206-208, base.py:109-162)
        zeros = numpy.zeros(model["pixels"].data.shape, dtype=model["pixels"].data.dtype)
        return model.copy(deep=True, pixels=zeros), numpy.zeros([nchan, npol])
    uvw = _device_uvw(bvis.uvw.data, device)
    # the visibilities, flags and weights (several times the uvw bytes) are
    # uploaded on a side stream while this stream builds the plan (bucket
    # sort); the gridding waits for them
    main = torch.cuda.current_stream(device)
    side = torch.cuda.Stream(device)
    side.wait_stream(main)
    with torch.cuda.stream(side):
        vis = None
        if not dopsf:
            vis = _to_device(bvis["vis"].data.reshape(R, vnchan, vnpol), cdt, device)
        flags = _to_device(bvis["flags"].data.reshape(R, vnchan, vnpol), None, device)
        if flags.dtype != torch.int64:
            flags = (flags != 0).to(torch.uint8)
        wgt = _to_device(bvis["imaging_weight"].data.reshape(R, vnchan, vnpol), rdt, device)
    uploaded = [t for t in (vis, flags, wgt) if t is not None]
    for t in uploaded:  # allocated on the side stream, used on this one
        t.record_stream(main)
    joined = [False]

    def join_uploads():
        if not joined[0]:
            main.wait_stream(side)
            joined[0] = True

    pdt = model["pixels"].data.dtype
    acc = torch.zeros((nchan, npol, ny, nx), dtype=torch.float64, device=device)
    sumwt = numpy.zeros([nchan, npol])
    mfs = nchan == 1 and vnchan > 1
    if mfs:
        groups = [(0, numpy.arange(vnchan))]
    else:
        groups = [(ic, numpy.nonzero(vis_to_im == ic)[0]) for ic in numpy.unique(vis_to_im)]
    for ichan, chans in groups:
        whole = len(chans) == vnchan
        f = torch.from_numpy(numpy.ascontiguousarray(freq[chans])).to(device)
        sel = None if whole else torch.from_numpy(chans).to(device)

        def pick(t):
            return t if (t is None or whole) else t[:, sel, :].contiguous()

        key, entry = _checkout_plan(uvw, f, nx, ny, pixsize, epsilon, do_wstacking, npol,
                                    precision, shift, _budget(kwargs))
        try:
            join_uploads()
            gvis = pick(vis)
            if residual_of is not None:
                img = _to_device(residual_of["pixels"].data[ichan], rdt, device)
                gvis = gvis - entry[1].dirty2ms(img, polmat=pred_pm, npol_vis=vnpol, layout="yx")
            dirty, sw = entry[1].ms2dirty(gvis, wgt=pick(wgt), flags=pick(flags),
                                          polmat=pm, psf=dopsf, layout="yx", sumwt=True)
            acc[ichan] += dirty
            sw = sw.cpu().numpy()
        finally:
            _checkin_plan(key, entry)
        sumwt[ichan] += sw
    if normalise:  # normalise_sumwt (imaging/base.py:109-162), on the device
        scale = numpy.where(sumwt > 0.0, 1.0 / numpy.where(sumwt > 0.0, sumwt, 1.0), 0.0)
        acc *= torch.from_numpy(scale).to(device)[:, :, None, None]
    # the new image: the model's metadata (deep-copied) with the dirty pixels
    pdt = _torch_dtype(pdt)
    im = model.copy(deep=True, pixels=_to_host(acc if acc.dtype == pdt else acc.to(pdt), pdt))
    return im, sumwt


# Names under which the dispatcher registers this backend.
predict_gb = predict_ng
invert_gb = invert_ng
