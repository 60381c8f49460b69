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
  channels that map to it (their sum is what ng.py accumulates).

Extra keyword arguments: ``precision`` ("fp64", the default, matches
the reference's complex128 path; "fp32" is the fast form), ``device``.
``threads`` and ``verbosity`` are accepted and ignored.
"""

import logging

import numpy
import torch

from ..data_models import copy_visibility
from ..polarisation import conversion_matrix
from ..wgridder import Plan
from .base import image_is_canonical, normalise_sumwt, shift_vis_to_image

log = logging.getLogger("rascil-logger")

__all__ = ["predict_ng", "invert_ng", "predict_gb", "invert_gb"]


def get_parameter(kwargs, key, default=None):
    """``rascil/data_models/parameters.py:108-125``: kwargs lookup with default."""
    if kwargs is None:
        return default
    value = kwargs.get(key, default)
    return default if value is None else value


def _vis_to_im(model, freq):
    return numpy.round(model.image_acc.wcs.sub([4]).wcs_world2pix(freq, 0)[0]).astype("int")


def _device_uvw(uvw, device, nan_to_num=False):
    u = torch.from_numpy(numpy.ascontiguousarray(uvw.reshape(-1, 3), dtype=numpy.float64))
    u = u.to(device)
    if nan_to_num:
        u = torch.nan_to_num(u)
    u[:, 0].neg_()
    u[:, 2].neg_()
    return u


def _to_device(x, dtype, device):
    return torch.from_numpy(numpy.ascontiguousarray(x)).to(device=device).to(dtype)


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

    newbvis = copy_visibility(bvis, zero=True)
    freq = numpy.asarray(bvis.frequency.data, dtype=numpy.float64)
    nrows, nbaselines, vnchan, vnpol = bvis.vis.shape
    m_nchan, m_npol, ny, nx = model["pixels"].data.shape
    assert m_npol == vnpol
    pixsize = abs(numpy.radians(model.image_acc.wcs.wcs.cdelt[0]))
    vis_to_im = _vis_to_im(model, freq)
    polmat = conversion_matrix(model.image_acc.polarisation_frame,
                               bvis.blockvisibility_acc.polarisation_frame)
    pm = None if numpy.array_equal(polmat, numpy.eye(vnpol)) else polmat
    uvw = _device_uvw(newbvis.uvw.data, device, nan_to_num=True)
    pixels = model["pixels"].data
    out = torch.empty((nrows * nbaselines, vnchan, vnpol), dtype=cdt, device=device)
    if m_nchan == 1:
        groups = [(0, numpy.arange(vnchan))]
    else:
        groups = [(ic, numpy.nonzero(vis_to_im == ic)[0]) for ic in numpy.unique(vis_to_im)]
    for ichan, chans in groups:
        f = torch.from_numpy(numpy.ascontiguousarray(freq[chans])).to(device)
        plan = Plan(uvw, f, nx, ny, pixsize, pixsize, epsilon, do_wstacking, npol=m_npol,
                    precision=precision)
        try:
            img = _to_device(pixels[ichan], rdt, device)
            vis = plan.dirty2ms(img, polmat=pm, npol_vis=vnpol, layout="yx")
        finally:
            plan.close()
        if len(chans) == vnchan:
            out = vis
        else:
            out[:, torch.from_numpy(chans).to(device), :] = vis
    result = out.reshape(nrows, nbaselines, vnchan, vnpol).cpu().numpy()
    if newbvis["vis"].data.dtype != result.dtype:
        result = result.astype(newbvis["vis"].data.dtype)
    newbvis["vis"].data = result
    return shift_vis_to_image(newbvis, model, tangent=True, inverse=True)


def invert_ng(bvis, model, dopsf=False, normalise=True, **kwargs):
    """Invert visibilities to (image, sumwt) (``ng.py:136-282``)."""
    assert image_is_canonical(model)
    im = model.copy(deep=True)
    epsilon = get_parameter(kwargs, "epsilon", 1e-12)
    do_wstacking = get_parameter(kwargs, "do_wstacking", True)
    precision = get_parameter(kwargs, "precision", "fp64")
    device = torch.device(get_parameter(kwargs, "device", "cuda"))
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    rdt = torch.float64 if precision == "fp64" else torch.float32

    sbvis = shift_vis_to_image(bvis, im, tangent=True, inverse=False)
    freq = numpy.asarray(sbvis.frequency.data, dtype=numpy.float64)
    nrows, nbaselines, vnchan, vnpol = sbvis.vis.shape
    nchan, npol, ny, nx = im["pixels"].data.shape
    pixsize = abs(numpy.radians(im.image_acc.wcs.wcs.cdelt[0]))
    polmat = conversion_matrix(bvis.blockvisibility_acc.polarisation_frame,
                               im.image_acc.polarisation_frame)
    pm = None if (npol == vnpol and numpy.array_equal(polmat, numpy.eye(vnpol))) else polmat
    vis_to_im = _vis_to_im(model, freq)
    R = nrows * nbaselines
    uvw = _device_uvw(sbvis.uvw.data, device)
    vis = None
    if not dopsf:
        vis = _to_device(sbvis["vis"].data.reshape(R, vnchan, vnpol), cdt, device)
    flags = torch.from_numpy(numpy.ascontiguousarray(
        sbvis["flags"].data.reshape(R, vnchan, vnpol))).to(device)
    if flags.dtype != torch.int64:
        flags = (flags != 0).to(torch.uint8)
    wgt = _to_device(sbvis["imaging_weight"].data.reshape(R, vnchan, vnpol), rdt, device)

    im["pixels"].data[...] = 0.0
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

        plan = Plan(uvw, f, nx, ny, pixsize, pixsize, epsilon, do_wstacking, npol=npol,
                    precision=precision)
        try:
            dirty, sw = plan.ms2dirty(pick(vis), wgt=pick(wgt), flags=pick(flags), polmat=pm,
                                      psf=dopsf, layout="yx", sumwt=True)
            dirty = dirty.cpu().numpy()
            sw = sw.cpu().numpy()
        finally:
            plan.close()
        im["pixels"].data[ichan] += dirty
        sumwt[ichan] += sw
    if normalise:
        im = normalise_sumwt(im, sumwt)
    return im, sumwt


# Names under which the dispatcher registers this backend.
predict_gb = predict_ng
invert_gb = invert_ng
