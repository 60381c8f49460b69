"""Pre/post steps of the ng path: canonical-image check, image phase
centre, phase rotation and sum-of-weights normalisation.

Restates ``rascil/processing_components/image/operations.py:75-102``
(``image_is_canonical``), ``rascil/processing_components/imaging/base.py:
67-137`` (``shift_vis_to_image``, ``normalise_sumwt``) and
``rascil/processing_components/visibility/base.py:296-357,1248-1264``
(tangent-plane ``phaserotate_visibility``) without astropy.
"""
import logging

import numpy

from ..data_models import SkyDirection, copy_visibility

log = logging.getLogger("rascil-logger")


def image_is_canonical(im):
    if im is None:
        return True
    w = im.image_acc.wcs.wcs
    ok = len(im["pixels"].data.shape) == 4
    ok = ok and w.ctype[0] == "RA---SIN" and w.ctype[1] == "DEC--SIN"
    ok = ok and w.ctype[2] == "STOKES"
    ok = ok and (w.ctype[3] == "FREQ" or w.ctype[3] == "MOMENT")
    return ok


def _ra_dec(direction):
    return float(direction.ra.rad), float(direction.dec.rad)


def lmn_of(direction, centre):
    """(l, m, n) of ``direction`` about ``centre`` (l east, m north)."""
    ra, dec = _ra_dec(direction)
    ra0, dec0 = _ra_dec(centre)
    dra = ra - ra0
    l = numpy.cos(dec) * numpy.sin(dra)
    m = numpy.sin(dec) * numpy.cos(dec0) - numpy.cos(dec) * numpy.sin(dec0) * numpy.cos(dra)
    n = numpy.sin(dec) * numpy.sin(dec0) + numpy.cos(dec) * numpy.cos(dec0) * numpy.cos(dra)
    return l, m, n


def image_phasecentre(im):
    """Sky direction of pixel (nx//2, ny//2) (0-relative) under the SIN
    projection of the image WCS (``imaging/base.py:87-89``)."""
    nchan, npol, ny, nx = im["pixels"].data.shape
    w = im.image_acc.wcs.wcs
    x = numpy.radians(w.cdelt[0] * (nx // 2 + 1 - w.crpix[0]))
    y = numpy.radians(w.cdelt[1] * (ny // 2 + 1 - w.crpix[1]))
    ra0, dec0 = numpy.radians(w.crval[0]), numpy.radians(w.crval[1])
    if x == 0.0 and y == 0.0:
        return SkyDirection(ra0, dec0)
    # SIN deprojection: intermediate (x, y) are the direction cosines (l, m),
    # l east-positive (cdelt[0] < 0 puts east to the left)
    l, m = x, y
    n = numpy.sqrt(1.0 - l * l - m * m)
    dec = numpy.arcsin(m * numpy.cos(dec0) + n * numpy.sin(dec0))
    ra = ra0 + numpy.arctan2(l, n * numpy.cos(dec0) - m * numpy.sin(dec0))
    return SkyDirection(ra, dec)


def separation(a, b):
    """Great-circle separation (rad), Vincenty form (accurate at tiny angles)."""
    ra1, d1 = _ra_dec(a)
    ra2, d2 = _ra_dec(b)
    dra = ra2 - ra1
    num = numpy.hypot(numpy.cos(d2) * numpy.sin(dra),
                      numpy.cos(d1) * numpy.sin(d2) - numpy.sin(d1) * numpy.cos(d2) * numpy.cos(dra))
    den = numpy.sin(d1) * numpy.sin(d2) + numpy.cos(d1) * numpy.cos(d2) * numpy.cos(dra)
    return float(numpy.arctan2(num, den))


def phase_rotation_needed(bvis, im):
    """As ``imaging/base.py:90``: rotate when the separation exceeds 1e-15 rad."""
    pc = image_phasecentre(im)
    return separation(bvis.phasecentre, pc) > 1e-15, pc


def phasor_direction(newphasecentre, phasecentre):
    """(l, m, sqrt(1 - l^2 - m^2) - 1) of ``newphasecentre`` about
    ``phasecentre`` (``visibility/base.py:1257-1258``), or None when the
    reference skips the rotation (``|n - 1| < 1e-15``, ``:311-314``)."""
    l, m, n = lmn_of(newphasecentre, phasecentre)
    if abs(n - 1.0) < 1e-15:
        return None
    return float(l), float(m), float(numpy.sqrt(1.0 - l * l - m * m) - 1.0)


def fused_phase_shift(bvis, im):
    """What ``shift_vis_to_image(bvis, im, tangent=True)`` does, as the
    gridder plan's fused phase shift: ``(rotates, shift)`` with ``shift`` in
    the plan's uvw frame (u and w negated, as ng.py hands uvw to the
    gridder).  ``rotates`` says whether the reference would re-label the
    visibilities' phase centre (the separation test of ``imaging/base.py:90``)."""
    needed, pc = phase_rotation_needed(bvis, im)
    if not needed:
        return False, (0.0, 0.0, 0.0)
    s = phasor_direction(pc, bvis.phasecentre)
    if s is None:
        return True, (0.0, 0.0, 0.0)
    return True, (-s[0], s[1], -s[2])


def _rotate_uvw(uvw, old, new):
    """uvw at phase centre ``old`` -> uvw at ``new`` through the XYZ frame
    (``visibility/base.py:331-355``: ``uvw_to_xyz`` with ha = -ra_old,
    ``xyz_to_uvw`` with ha = -ra_new); rotations of [R][3] coordinates."""
    from ..simulation import xyz_to_uvw
    ra0, dec0 = _ra_dec(old)
    ra1, dec1 = _ra_dec(new)
    u, v, w = uvw[:, 0], uvw[:, 1], uvw[:, 2]
    h, d = -ra0, dec0
    # inverse of xyz_to_uvw(., h, d)
    z = w * numpy.sin(d) + v * numpy.cos(d)
    v0 = v * numpy.sin(d) - w * numpy.cos(d)
    x = u * numpy.cos(h) + v0 * numpy.sin(h)
    y = v0 * numpy.cos(h) - u * numpy.sin(h)
    return xyz_to_uvw(numpy.stack([x, y, z], axis=-1), -ra1, dec1)


def phaserotate_visibility(vis, newphasecentre, tangent=True, inverse=False, **kwargs):
    """Phase-rotate to a new phase centre (``visibility/base.py:296-357``):
    a copy whose visibilities are multiplied, on the GPU
    (``gb_phase_rotate``), by conj(phasor) (or by the phasor if
    ``inverse``), phasor = exp(-2 pi i uvw_lambda . s).  With
    ``tangent=False`` the uvw are also rotated to the new phase centre and
    the copy's phase centre updated, as the reference does."""
    s = phasor_direction(newphasecentre, vis.phasecentre)
    if s is None:
        return vis
    import torch

    from .. import _lib
    data = vis["vis"].data
    if data.dtype == numpy.complex128:
        prec, cdt = _lib.GB_FP64, torch.complex128
    elif data.dtype == numpy.complex64:
        prec, cdt = _lib.GB_FP32, torch.complex64
    else:
        raise TypeError("vis must be complex64 or complex128, not %s" % data.dtype)
    nrows, nbl, nchan, npol = data.shape
    device = torch.device(kwargs.get("device", "cuda"))

    def up(x):
        t = torch.from_numpy(numpy.ascontiguousarray(x))
        return t.to(device=device, non_blocking=t.is_pinned())

    with torch.cuda.device(device):
        dv = up(data)
        uvw = up(numpy.asarray(vis.uvw.data, dtype=numpy.float64).reshape(-1, 3))
        freq = up(numpy.asarray(vis.frequency.data, dtype=numpy.float64))
        stream = torch.cuda.current_stream(device).cuda_stream
        _lib.check(_lib.load().gb_phase_rotate(
            uvw.data_ptr(), freq.data_ptr(), nrows * nbl, nchan, npol, dv.data_ptr(), prec,
            s[0], s[1], s[2], 1 if inverse else 0, stream), "phaserotate_visibility")
        host = torch.empty(dv.shape, dtype=cdt, pin_memory=True)
        host.copy_(dv)
    newvis = copy_visibility(vis, vis=host.numpy())
    if not tangent:
        uvw = numpy.asarray(vis.uvw.data, dtype=numpy.float64).reshape(-1, 3)
        newvis["uvw"].data[...] = _rotate_uvw(uvw, vis.phasecentre,
                                              newphasecentre).reshape(vis.uvw.data.shape)
        newvis.attrs["phasecentre"] = newphasecentre
    return newvis


def shift_vis_to_image(bvis, im, tangent=True, inverse=False, **kwargs):
    """Phase-rotate vis to the image phase centre, or back if ``inverse``
    (``imaging/base.py:67-106``).  invert_ng / predict_ng fuse this step
    into the gridder (``fused_phase_shift``); this is the standalone form."""
    needed, pc = phase_rotation_needed(bvis, im)
    if needed:
        bvis = phaserotate_visibility(bvis, pc, tangent=tangent, inverse=inverse, **kwargs)
        bvis.attrs["phasecentre"] = im.image_acc.phasecentre
    return bvis


def normalise_sumwt(im, sumwt):
    """Divide each (chan, pol) plane by sumwt, zero it where sumwt <= 0."""
    nchan, npol, _, _ = im["pixels"].data.shape
    assert sumwt is not None
    for chan in range(nchan):
        for pol in range(npol):
            if sumwt[chan, pol] > 0.0:
                im["pixels"].data[chan, pol] = im["pixels"].data[chan, pol] / sumwt[chan, pol]
            else:
                im["pixels"].data[chan, pol] = 0.0
    return im
