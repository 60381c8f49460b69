"""List workflows of the ng path on one GPU.

RASCIL images a list of visibility blocks (frequency windows, snapshots) by
running one ``invert_blockvisibility`` / ``predict_blockvisibility`` task
per block through Dask and then summing the results
(``rascil/workflows/rsexecute/imaging/imaging_rsexecute.py:72-181,844-931``,
``rascil/processing_components/imaging/imaging_helpers.py:17-72``).  Here
the same functions, with the same arguments, results and side effects, run
the blocks concurrently on one GPU:

* a pool of worker threads, each with its own CUDA stream, takes the blocks
  in order; one block's transfers, bucket sort, gridding and transforms
  overlap another's (ctypes and torch release the GIL while they wait);
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


def invert_list_rsexecute_workflow(vis_list, template_model_imagelist, context, dopsf=False,
                                   normalise=True, **kwargs):
    """One (image, sumwt) per block (``imaging_rsexecute.py:115-157``).
    Extra keyword: ``streams`` (concurrent blocks, default 4)."""
    if not isinstance(template_model_imagelist, collections.abc.Iterable):
        template_model_imagelist = [template_model_imagelist]
    template_model_imagelist = list(template_model_imagelist)
    assert len(template_model_imagelist) == len(vis_list)
    nstreams = _streams(kwargs)

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
    nstreams = _streams(kwargs)
    vis_list = zero_list_rsexecute_workflow(vis_list, copy=False)
    model_imagelist = list(model_imagelist)
    assert len(model_imagelist) == len(vis_list)

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
