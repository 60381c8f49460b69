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

from ..data_models import SPEED_OF_LIGHT, SkyDirection, copy_visibility

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


def shift_vis_to_image(bvis, im, tangent=True, inverse=False):
    """Phase-rotate vis to the image phase centre (or back if ``inverse``)."""
    if not tangent:
        raise NotImplementedError("only tangent-plane rotation is supported")
    needed, pc = phase_rotation_needed(bvis, im)
    if not needed:
        return bvis
    l, m, n = lmn_of(pc, bvis.phasecentre)
    if abs(n - 1.0) < 1e-15 and abs(l) < 1e-15 and abs(m) < 1e-15:
        return bvis
    new = copy_visibility(bvis)
    s = numpy.array([l, m, n - 1.0])
    f = new.frequency.data / SPEED_OF_LIGHT
    phase = numpy.einsum("tbs,s->tb", new.uvw.data, s)[..., None] * f
    phasor = numpy.exp(-2j * numpy.pi * phase)[..., None]
    if inverse:
        new["vis"].data = new["vis"].data * phasor
    else:
        new["vis"].data = new["vis"].data * numpy.conj(phasor)
    new.attrs["phasecentre"] = im.image_acc.phasecentre
    return new


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
