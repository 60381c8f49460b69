"""List workflows of the ng path on one GPU.

RASCIL images a list of visibility blocks (frequency windows, snapshots) by
running one ``invert_blockvisibility`` / ``predict_blockvisibility`` task
per block through Dask and then summing the results
(``rascil/workflows/rsexecute/imaging/imaging_rsexecute.py:72-181,844-931``,
``rascil/processing_components/imaging/imaging_helpers.py:17-72``).  Here
the same functions, with the same arguments, results and side effects, run
the blocks on one GPU:

* ``invert_list`` / ``predict_list`` over blocks whose visibility channels
  all map to one image channel (MFS images, or one channel per block) run
  as ONE device program (``gb_batch_run_items``): every block's arrays are
  uploaded, one plan per block, then rounds over workspace slots in which
  the gridding (or degridding) of every slot's block runs in one persistent
  launch fed from a device work queue, with each block's transforms on its
  slot's stream;
* other lists (several image channels per block) run on a pool of worker
  threads, each with its own CUDA stream; one block's transfers, bucket
  sort, gridding and transforms overlap another's (ctypes and torch release
  the GIL while they wait);
* the residual workflow runs each block's predict, subtraction and invert
  on the device in one pass (``residual_ng``), so the model visibilities
  never travel to the host and back;
* ``sum_invert_results`` forms the sumwt-weighted image sum on the device
  in FP64.

``rsexecute`` is a stand-in for RASCIL's execution wrapper with Dask off
(``execution_support/rsexecute.py``: ``execute`` calls the function,
``compute`` / ``persist`` / ``optimize`` return their argument), so code
written against the reference's workflows runs unchanged.
"""
import collections.abc
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy
import torch

from .data_models import copy_visibility
from .imaging.imaging import invert_blockvisibility, predict_blockvisibility
from .imaging.ng import _to_device, _to_host, _torch_dtype, residual_ng

__all__ = ["rsexecute", "invert_list_rsexecute_workflow", "predict_list_rsexecute_workflow",
           "residual_list_rsexecute_workflow", "zero_list_rsexecute_workflow",
           "subtract_list_rsexecute_workflow", "sum_invert_results",
           "sum_invert_results_rsexecute", "sum_predict_results",
           "sum_predict_results_rsexecute", "remove_sumwt"]

DEFAULT_STREAMS = 4
# Per-block memory for one batch of w-planes when blocks run concurrently
# (each block's plan holds one batch; the library default of 32 GiB is sized
# for one large problem on its own).
CONCURRENT_GRID_BUDGET = 4 << 30


class _Rsexecute:
    """RASCIL's rsexecute with Dask off: calls run immediately."""

    using_dask = False

    def execute(self, func, *args, **kwargs):
        return func

    def compute(self, value, sync=False):
        return value

    def persist(self, graph, **kwargs):
        return graph

    def optimize(self, *args, **kwargs):
        return args[0] if len(args) == 1 else args

    def scatter(self, graph, **kwargs):
        return graph

    def gather(self, graph):
        return graph

    def set_client(self, *args, **kwargs):
        return None

    def close(self):
        return None

    def type(self):
        return "function"


rsexecute = _Rsexecute()


def _streams(kwargs):
    n = int(kwargs.pop("streams", DEFAULT_STREAMS))
    if n > 1:
        kwargs.setdefault("grid_budget_bytes", CONCURRENT_GRID_BUDGET)
    return n


def _map_blocks(func, items, nstreams):
    """[func(x) for x in items], run by up to ``nstreams`` worker threads,
    each issuing its GPU work on its own CUDA stream.  ``func`` returns host
    results (the ng functions end with a synchronous device-to-host copy),
    so nothing is left pending on a worker stream when the map returns.
    The first exception is re-raised after every block has finished."""
    items = list(items)
    if nstreams <= 1 or len(items) <= 1 or not torch.cuda.is_available():
        return [func(x) for x in items]
    device = torch.device("cuda", torch.cuda.current_device())
    origin = torch.cuda.current_stream(device)
    local = threading.local()

    def run(x):
        stream = getattr(local, "stream", None)
        if stream is None:
            stream = local.stream = torch.cuda.Stream(device=device)
            stream.wait_stream(origin)  # work the caller queued before the map
        with torch.cuda.device(device), torch.cuda.stream(stream):
            return func(x)

    with ThreadPoolExecutor(max_workers=min(nstreams, len(items))) as pool:
        return list(pool.map(run, items))


# ---------------------------------------------------------------------------
# the list as one device program (gb_batch_run_items)

def _single_group(bvis, model):
    """The image channel all of the block's visibility channels map to (the
    block then needs one plan, as the device program takes), else None."""
    from .imaging.ng import _vis_to_im
    freq = numpy.asarray(bvis.frequency.data, dtype=numpy.float64)
    nchan = model["pixels"].data.shape[0]
    if nchan == 1:
        return 0
    v2i = numpy.unique(_vis_to_im(model, freq))
    return int(v2i[0]) if len(v2i) == 1 else None


def _batchable(vis_list, models, context):
    if context not in ("ng", "gb", "2d") or not torch.cuda.is_available() or len(vis_list) < 2:
        return False
    for bvis, model in zip(vis_list, models):
        if bvis is None or model is None:
            return False
        nrows, nbl, vnchan, _ = bvis.vis.shape
        if nrows * nbl == 0 or vnchan == 0 or _single_group(bvis, model) is None:
            return False
        if not numpy.isfinite(numpy.asarray(bvis.uvw.data)).all():
            return False
    return True


def _run_program(plans, items, nslots, device):
    """gb_batch_run_items over the plans on nslots workspace slots and
    streams, ordered after (and before) the current stream's work."""
    import ctypes

    from . import _lib
    n = len(plans)
    nslots = max(1, min(nslots, n, 16))
    need = [256] * nslots
    for i, p in enumerate(plans):
        need[i % nslots] = max(need[i % nslots], p.workspace_bytes)
    workspaces = [torch.empty(b, dtype=torch.uint8, device=device) for b in need]
    origin = torch.cuda.current_stream(device)
    streams = [origin] + [torch.cuda.Stream(device=device) for _ in range(nslots - 1)]
    for st in streams[1:]:
        st.wait_stream(origin)
    ptrs = (ctypes.c_void_p * n)(*[p._handle.value for p in plans])
    arr = (_lib.BatchItem * n)(*items)
    ws = (ctypes.c_void_p * nslots)(*[w.data_ptr() for w in workspaces])
    wsb = (ctypes.c_size_t * nslots)(*[w.numel() for w in workspaces])
    sts = (ctypes.c_void_p * nslots)(*[st.cuda_stream for st in streams])
    with torch.cuda.device(device):
        _lib.check(_lib.load().gb_batch_run_items(ptrs, arr, n, ws, wsb, sts, nslots,
                                                  _lib.GB_LAYOUT_YX), "gb_batch_run_items")
    for w in workspaces:  # the allocator must not recycle them under pending work
        for st in streams:
            w.record_stream(st)
    for p, i in zip(plans, range(n)):
        p.workspace = workspaces[i % nslots]


def _polmat_ptr(m, keep):
    import ctypes
    if m is None:
        return None
    flat = numpy.ascontiguousarray(numpy.asarray(m, dtype=numpy.complex128).view(numpy.float64)
                                   .ravel())
    keep.append(flat)
    return flat.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _invert_list_program(vis_list, models, dopsf, normalise, kwargs, nslots):
    """invert_ng of every block (one plan each) as one device program."""
    from . import _lib
    from .imaging.base import fused_phase_shift
    from .imaging.ng import _budget, _device_uvw, _to_device, _to_host, get_parameter
    from .polarisation import conversion_matrix
    from .wgridder import Plan
    epsilon = get_parameter(kwargs, "epsilon", 1e-12)
    do_wstacking = get_parameter(kwargs, "do_wstacking", True)
    precision = get_parameter(kwargs, "precision", "fp64")
    device = torch.device(get_parameter(kwargs, "device", "cuda"))
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    rdt = torch.float64 if precision == "fp64" else torch.float32
    plans, items, outs, keep = [], [], [], []
    try:
        for bvis, model in zip(vis_list, models):
            _, shift = fused_phase_shift(bvis, model)
            freq = numpy.asarray(bvis.frequency.data, dtype=numpy.float64)
            nrows, nbaselines, vnchan, vnpol = bvis.vis.shape
            nchan, npol, ny, nx = model["pixels"].data.shape
            R = nrows * nbaselines
            pixsize = abs(numpy.radians(model.image_acc.wcs.wcs.cdelt[0]))
            polmat = conversion_matrix(bvis.blockvisibility_acc.polarisation_frame,
                                       model.image_acc.polarisation_frame)
            pm = None if (npol == vnpol and numpy.array_equal(polmat, numpy.eye(vnpol))) \
                else polmat
            uvw = _device_uvw(bvis.uvw.data, device)
            f = torch.from_numpy(freq.copy()).to(device)
            vis = None if dopsf else _to_device(bvis["vis"].data.reshape(R, vnchan, vnpol), cdt,
                                                device)
            flags = _to_device(bvis["flags"].data.reshape(R, vnchan, vnpol), None, device)
            if flags.dtype != torch.int64:
                flags = (flags != 0).to(torch.uint8)
            wgt = _to_device(bvis["imaging_weight"].data.reshape(R, vnchan, vnpol), rdt, device)
            plan = Plan(uvw, f, nx, ny, pixsize, pixsize, epsilon, do_wstacking, npol=npol,
                        precision=precision, bind=False, phase_shift=shift,
                        grid_budget_bytes=_budget(kwargs))
            plans.append(plan)
            dirty = torch.empty((npol, ny, nx), dtype=rdt, device=device)
            sumwt = torch.empty(npol, dtype=torch.float64, device=device)
            keep.append((uvw, f, vis, flags, wgt))
            items.append(_lib.BatchItem(
                vis=None if vis is None else vis.data_ptr(), npol_vis=vnpol,
                psf=1 if dopsf else 0, wgt=wgt.data_ptr(), flags=flags.data_ptr(),
                flags_type=_lib.GB_FLAGS_I64 if flags.dtype == torch.int64 else _lib.GB_FLAGS_U8,
                polmat_in=_polmat_ptr(pm, keep), dirty=dirty.data_ptr(),
                sumwt=sumwt.data_ptr(), model=None, polmat_out=None, npol_out=npol, pred=None))
            outs.append((dirty, sumwt))
        _run_program(plans, items, nslots, device)
        results = []
        for (dirty, sw), bvis, model in zip(outs, vis_list, models):
            ichan = _single_group(bvis, model)
            nchan, npol, ny, nx = model["pixels"].data.shape
            acc = torch.zeros((nchan, npol, ny, nx), dtype=torch.float64, device=device)
            acc[ichan] = dirty
            sumwt = numpy.zeros([nchan, npol])
            sumwt[ichan] = sw.cpu().numpy()
            if normalise:  # normalise_sumwt (imaging/base.py:109-162), on the device
                scale = numpy.where(sumwt > 0.0, 1.0 / numpy.where(sumwt > 0.0, sumwt, 1.0), 0.0)
                acc *= torch.from_numpy(scale).to(device)[:, :, None, None]
            pdt = _torch_dtype(model["pixels"].data.dtype)
            im = model.copy(deep=True,
                            pixels=_to_host(acc if acc.dtype == pdt else acc.to(pdt), pdt))
            results.append((im, sumwt))
        return results
    finally:
        torch.cuda.current_stream(device).synchronize()
        for p in plans:
            p.close()


def _predict_list_program(vis_list, models, kwargs, nslots):
    """predict_ng of every block (one plan each) as one device program."""
    from . import _lib
    from .imaging.base import fused_phase_shift
    from .imaging.ng import _budget, _device_uvw, _to_device, _to_host, get_parameter
    from .polarisation import conversion_matrix
    from .wgridder import Plan
    epsilon = get_parameter(kwargs, "epsilon", 1e-12)
    do_wstacking = get_parameter(kwargs, "do_wstacking", True)
    precision = get_parameter(kwargs, "precision", "fp64")
    device = torch.device(get_parameter(kwargs, "device", "cuda"))
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    rdt = torch.float64 if precision == "fp64" else torch.float32
    plans, items, outs, keep = [], [], [], []
    try:
        for bvis, model in zip(vis_list, models):
            rotates, shift = fused_phase_shift(bvis, model)
            freq = numpy.asarray(bvis.frequency.data, dtype=numpy.float64)
            nrows, nbaselines, vnchan, vnpol = bvis.vis.shape
            m_nchan, m_npol, ny, nx = model["pixels"].data.shape
            assert m_npol == vnpol
            pixsize = abs(numpy.radians(model.image_acc.wcs.wcs.cdelt[0]))
            polmat = conversion_matrix(model.image_acc.polarisation_frame,
                                       bvis.blockvisibility_acc.polarisation_frame)
            pm = None if numpy.array_equal(polmat, numpy.eye(vnpol)) else polmat
            uvw = _device_uvw(bvis.uvw.data, device, nan_to_num=True)
            f = torch.from_numpy(freq.copy()).to(device)
            ichan = _single_group(bvis, model)
            img = _to_device(model["pixels"].data[ichan], rdt, device)
            plan = Plan(uvw, f, nx, ny, pixsize, pixsize, epsilon, do_wstacking, npol=m_npol,
                        precision=precision, bind=False, phase_shift=shift,
                        grid_budget_bytes=_budget(kwargs))
            plans.append(plan)
            out = torch.empty((nrows * nbaselines, vnchan, vnpol), dtype=cdt, device=device)
            keep.append((uvw, f, img))
            items.append(_lib.BatchItem(vis=None, npol_vis=m_npol, psf=0, wgt=None, flags=None,
                                        flags_type=0, polmat_in=None, dirty=None, sumwt=None,
                                        model=img.data_ptr(), polmat_out=_polmat_ptr(pm, keep),
                                        npol_out=vnpol, pred=out.data_ptr()))
            outs.append((out, rotates))
        _run_program(plans, items, nslots, device)
        results = []
        for (out, rotates), bvis, model in zip(outs, vis_list, models):
            vdt = bvis["vis"].data.dtype
            nrows, nbaselines, vnchan, vnpol = bvis.vis.shape
            o = out.reshape(nrows, nbaselines, vnchan, vnpol)
            want = torch.complex128 if vdt == numpy.complex128 else torch.complex64
            if o.dtype != want:
                o = o.to(want)
            result = _to_host(o, o.dtype)
            if result.dtype != vdt:
                result = result.astype(vdt)
            newbvis = copy_visibility(bvis, vis=result)
            if rotates:
                newbvis.attrs["phasecentre"] = model.image_acc.phasecentre
            results.append(newbvis)
        return results
    finally:
        torch.cuda.current_stream(device).synchronize()
        for p in plans:
            p.close()


def invert_list_rsexecute_workflow(vis_list, template_model_imagelist, context, dopsf=False,
                                   normalise=True, **kwargs):
    """One (image, sumwt) per block (``imaging_rsexecute.py:115-157``).
    Extra keywords: ``streams`` (workspace slots of the device program, or
    concurrent blocks on worker threads, default 4), ``program`` (False:
    always the worker-thread map)."""
    if not isinstance(template_model_imagelist, collections.abc.Iterable):
        template_model_imagelist = [template_model_imagelist]
    template_model_imagelist = list(template_model_imagelist)
    assert len(template_model_imagelist) == len(vis_list)
    program = kwargs.pop("program", True)
    nstreams = _streams(kwargs)
    if program and _batchable(vis_list, template_model_imagelist, context):
        kw = dict(kwargs)
        if context == "2d":
            kw["do_wstacking"] = False
        return _invert_list_program(vis_list, template_model_imagelist, dopsf, normalise, kw,
                                    max(nstreams, 1))

    def one(i):
        return invert_blockvisibility(vis_list[i], template_model_imagelist[i], dopsf=dopsf,
                                      normalise=normalise, context=context, **kwargs)

    return _map_blocks(one, range(len(vis_list)), nstreams)


def zero_list_rsexecute_workflow(vis_list, copy=True):
    """Zeroed copies, or the blocks zeroed in place (``:844-866``)."""
    out = []
    for vis in vis_list:
        if vis is None:
            out.append(None)
        elif copy:
            out.append(copy_visibility(vis, zero=True))
        else:
            vis["vis"].data[...] = 0.0
            out.append(vis)
    return out


def predict_list_rsexecute_workflow(vis_list, model_imagelist, context, **kwargs):
    """Predicted copies of the blocks (``:72-112``).  As in the reference,
    the input blocks' visibilities are zeroed in place first."""
    program = kwargs.pop("program", True)
    nstreams = _streams(kwargs)
    vis_list = zero_list_rsexecute_workflow(vis_list, copy=False)
    model_imagelist = list(model_imagelist)
    assert len(model_imagelist) == len(vis_list)
    if program and _batchable(vis_list, model_imagelist, context):
        kw = dict(kwargs)
        if context == "2d":
            kw["do_wstacking"] = False
        return _predict_list_program(vis_list, model_imagelist, kw, max(nstreams, 1))

    def one(i):
        return predict_blockvisibility(vis_list[i], model_imagelist[i], context=context,
                                       **kwargs)

    return _map_blocks(one, range(len(vis_list)), nstreams)


def subtract_list_rsexecute_workflow(vis_list, model_vislist):
    """Copies of the blocks minus the model blocks (``:869-892``)."""
    out = []
    for vis, model in zip(vis_list, model_vislist):
        if vis is None or model is None:
            out.append(None)
            continue
        assert vis.vis.shape == model.vis.shape
        out.append(copy_visibility(vis, vis=vis["vis"].data - model["vis"].data))
    return out


def residual_list_rsexecute_workflow(vis, model_imagelist, context="2d", **kwargs):
    """(residual image, sumwt) per block (``:160-181``): the invert of each
    block minus its model's prediction, normalised, in one device pass per
    block."""
    if context not in ("ng", "gb", "2d"):
        raise ValueError(f"Unknown imaging context {context}")
    if context == "2d":
        kwargs["do_wstacking"] = False
    nstreams = _streams(kwargs)
    model_imagelist = list(model_imagelist)
    assert len(model_imagelist) == len(vis)

    def one(i):
        return residual_ng(vis[i], model_imagelist[i], normalise=True, **kwargs)

    return _map_blocks(one, range(len(vis)), nstreams)


def sum_invert_results(image_list, device="cuda"):
    """Sumwt-weighted sum of (image, sumwt) pairs, normalised by the summed
    sumwt (``imaging_helpers.py:17-42``): a copy for one pair; otherwise
    sum_i sumwt_i image_i / sum_i sumwt_i per (channel, pol), zero where the
    summed sumwt is not positive, accumulated in FP64 on the GPU.  ``None``
    entries are skipped, as in the reference."""
    if len(image_list) == 1:
        return image_list[0][0].copy(deep=True), image_list[0][1]
    first = image_list[0][0]
    device = torch.device(device)
    acc = torch.zeros(first["pixels"].data.shape, dtype=torch.float64, device=device)
    sumwt = numpy.zeros_like(numpy.asarray(image_list[0][1], dtype=numpy.float64))
    for arg in image_list:
        if arg is None:
            continue
        w = numpy.asarray(arg[1], dtype=numpy.float64)
        pixels = _to_device(arg[0]["pixels"].data, torch.float64, device)
        acc += torch.from_numpy(w).to(device)[..., None, None] * pixels
        sumwt += w
    scale = numpy.where(sumwt > 0.0, 1.0 / numpy.where(sumwt > 0.0, sumwt, 1.0), 0.0)
    acc *= torch.from_numpy(scale).to(device)[..., None, None]
    pdt = _torch_dtype(first["pixels"].data.dtype)
    im = first.copy(deep=True, pixels=_to_host(acc if acc.dtype == pdt else acc.to(pdt), pdt))
    return im, sumwt


def sum_invert_results_rsexecute(image_list):
    """The same sum (``imaging_rsexecute.py:913-930`` reduces it as a tree;
    the result is the weighted mean either way)."""
    return sum_invert_results(image_list)


def remove_sumwt(results):
    """The images of (image, sumwt) pairs (``imaging_helpers.py:45-54``)."""
    try:
        return [d[0] for d in results]
    except KeyError:
        return results


def sum_predict_results(results):
    """Sum of predicted blocks into the first one (``imaging_helpers.py:57-72``;
    the first non-None block is updated in place and returned)."""
    total = None
    for result in results:
        if result is None:
            continue
        if total is None:
            total = result
        else:
            assert total["vis"].data.shape == result["vis"].data.shape
            total["vis"].data += result["vis"].data
    return total


def sum_predict_results_rsexecute(bvis_list, split=2):
    """The same sum (``imaging_rsexecute.py:895-910``)."""
    return sum_predict_results(bvis_list)
