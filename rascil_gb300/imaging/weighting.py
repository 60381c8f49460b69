"""Imaging weights on the GPU: RASCIL's ``weight_visibility``.

Same signature, arguments and result as
``rascil/processing_components/imaging/weighting.py:27-48``
(``weight_visibility(vis, model, weighting="uniform", robustness=0.0)``;
``weight_blockvisibility`` ``:51-64`` is its deprecated alias).  The
arithmetic of ``grid_blockvisibility_weight_to_griddata`` and
``griddata_blockvisibility_reweight`` (``griddata/gridding.py:260-425``)
runs in ``gb_weight_visibility`` (``csrc/gb_weight.cu``): the flagged imaging
weights gridded with FP64 atomics onto the image-sized uv grid, then every
sample reweighted (uniform, robust or natural).  Like the reference, the new
imaging weights are written into ``vis["imaging_weight"]`` in place and
``vis`` is returned; a sample outside the grid raises (``OutOfGridError``,
an ``AssertionError`` as the reference's assert).
"""
import ctypes

import numpy
import torch

from .. import _lib
from .base import image_is_canonical

__all__ = ["weight_visibility", "weight_blockvisibility"]

_SCHEMES = {"natural": _lib.GB_WEIGHT_NATURAL, "uniform": _lib.GB_WEIGHT_UNIFORM,
            "robust": _lib.GB_WEIGHT_ROBUST}


def _dev(x, dtype, device):
    t = torch.from_numpy(numpy.ascontiguousarray(x))
    t = t.to(device=device, non_blocking=t.is_pinned())
    return t if dtype is None else t.to(dtype)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def weight_visibility(vis, model, weighting="uniform", robustness=0.0, **kwargs):
    """Weight the visibility data (``weighting.py:27-48``).

    :param vis: BlockVisibility
    :param model: canonical Image giving the uv grid (its size and cellsize)
    :param weighting: "uniform", "robust" or "natural"
    :param robustness: Briggs robustness (robust only)
    :return: vis with ``imaging_weight`` replaced
    """
    assert image_is_canonical(model)
    if weighting not in _SCHEMES:
        raise AssertionError("Weighting {} not supported".format(weighting))
    device = torch.device(kwargs.get("device", "cuda"))
    nrows, nbl, nchan, npol = vis.vis.shape
    nchan_img, _, ny, nx = model["pixels"].data.shape
    freq = numpy.asarray(vis.frequency.data, dtype=numpy.float64)
    wcs = model.image_acc.wcs
    vis_to_im = numpy.round(wcs.sub([4]).wcs_world2pix(freq, 0)[0]).astype(numpy.int64)
    # numpy indexing in the reference: negative channels count from the end,
    # anything else outside the image's channels raises
    bad = (vis_to_im >= nchan_img) | (vis_to_im < -nchan_img)
    if bad.any():
        raise IndexError("visibility channel %d maps to image channel %d of %d"
                         % (int(numpy.argmax(bad)), int(vis_to_im[bad][0]), nchan_img))
    vis_to_im = numpy.where(vis_to_im < 0, vis_to_im + nchan_img, vis_to_im).astype(numpy.int32)
    cdelt = wcs.wcs.cdelt
    R = nrows * nbl
    if R == 0 or nchan == 0 or npol == 0:
        return vis  # no samples: nothing gridded, nothing reweighted
    lib = _lib.load()
    with torch.cuda.device(device):
        uvw = _dev(vis.uvw.data.reshape(R, 3), torch.float64, device)
        f = _dev(freq, torch.float64, device)
        v2i = _dev(vis_to_im, torch.int32, device)
        wgt = _dev(vis["weight"].data.reshape(R, nchan, npol), torch.float64, device)
        imw = _dev(vis["imaging_weight"].data.reshape(R, nchan, npol), torch.float64, device)
        flags = _dev(vis["flags"].data.reshape(R, nchan, npol), None, device)
        if flags.dtype == torch.int64:
            ftype = _lib.GB_FLAGS_I64
        else:
            flags = (flags != 0).to(torch.uint8)
            ftype = _lib.GB_FLAGS_U8
        grid = torch.empty((nchan_img, ny, nx, npol), dtype=torch.float64, device=device)
        cells = torch.empty((R, nchan), dtype=torch.int32, device=device)
        out = torch.empty((R, nchan, npol), dtype=torch.float64, device=device)
        sums = torch.empty(2, dtype=torch.float64, device=device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
        _lib.check(lib.gb_weight_visibility(
            _ptr(uvw), _ptr(f), R, nchan, npol, _ptr(v2i), nchan_img, nx, ny,
            float(cdelt[0]), float(cdelt[1]), _ptr(wgt), _ptr(imw), _ptr(flags), ftype,
            _SCHEMES[weighting], float(robustness), _ptr(grid), _ptr(cells), _ptr(out), _ptr(sums),
            stream),
            "weight_visibility")
        dst = vis["imaging_weight"].data
        res = out.reshape(dst.shape)
        ddt = torch.from_numpy(numpy.zeros(0, dtype=dst.dtype)).dtype
        if res.dtype != ddt:
            res = res.to(ddt)
        if dst.flags.c_contiguous and dst.flags.writeable:
            # straight into the caller's array (a DMA when it is page-locked)
            torch.from_numpy(dst).copy_(res)
        else:
            dst[...] = res.cpu().numpy()
    return vis


def weight_blockvisibility(vis, model, weighting="uniform", robustness=0.0, **kwargs):
    """Deprecated alias of :func:`weight_visibility` (``weighting.py:51-64``)."""
    return weight_visibility(vis, model, weighting, robustness, **kwargs)
