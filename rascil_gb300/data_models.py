"""Slim ``BlockVisibility`` / ``Image`` with the attribute surface the ng
imaging path uses.

RASCIL's data models (``rascil/data_models/memory_data_models.py:511-720``
Image, ``:1214-1529`` BlockVisibility) are xarray Datasets with astropy
WCS and SkyCoord members.  The imaging functions here touch only:

* bvis: ``bvis["vis"].data``, ``bvis.vis.shape``, ``bvis.uvw.data``,
  ``bvis.frequency.data``, ``bvis.phasecentre`` (``.ra.rad``, ``.dec.rad``),
  ``bvis.blockvisibility_acc.{flagged_vis, flagged_imaging_weight,
  polarisation_frame}``, ``bvis.attrs``;
* model: ``model["pixels"].data`` [nchan, npol, ny, nx],
  ``model.image_acc.{wcs, polarisation_frame, phasecentre, shape}``,
  ``model.copy(deep=True)``.

The classes below provide exactly that surface on numpy arrays, so the
imaging functions accept either these or RASCIL's own objects.
"""

import copy
import os
from concurrent.futures import ThreadPoolExecutor

import numpy

from .polarisation import PolarisationFrame

SPEED_OF_LIGHT = 299792458.0


class _Angle:
    __slots__ = ("rad",)

    def __init__(self, rad):
        self.rad = float(rad)

    @property
    def deg(self):
        return numpy.degrees(self.rad)


class SkyDirection:
    """Minimal sky direction (ICRS ra/dec in radians) with ``.ra.rad``."""

    def __init__(self, ra, dec):
        self.ra = _Angle(ra)
        self.dec = _Angle(dec)

    def separation_rad(self, other):
        """Great-circle separation in radians (Vincenty form)."""
        ra1, d1 = self.ra.rad, self.dec.rad
        ra2, d2 = other.ra.rad, other.dec.rad
        dra = ra2 - ra1
        num = numpy.hypot(numpy.cos(d2) * numpy.sin(dra),
                          numpy.cos(d1) * numpy.sin(d2) - numpy.sin(d1) * numpy.cos(d2) * numpy.cos(dra))
        den = numpy.sin(d1) * numpy.sin(d2) + numpy.cos(d1) * numpy.cos(d2) * numpy.cos(dra)
        return float(numpy.arctan2(num, den))

    def __repr__(self):
        return "SkyDirection(ra=%.9f rad, dec=%.9f rad)" % (self.ra.rad, self.dec.rad)


_PARALLEL_MIN_BYTES = 64 << 20


def parallel_copy(a):
    """Copy of a numpy array; large C-contiguous arrays are copied in
    os.cpu_count() slices on threads (numpy.copyto releases the GIL), which
    matters for the multi-GB visibility, flag and weight arrays."""
    a = numpy.asarray(a)
    if a.nbytes < _PARALLEL_MIN_BYTES or not a.flags.c_contiguous:
        return a.copy()
    out = numpy.empty_like(a)
    src, dst = a.reshape(-1), out.reshape(-1)
    nthreads = max(1, min(32, os.cpu_count() or 1))
    step = -(-src.size // nthreads)

    def part(i):
        numpy.copyto(dst[i * step:(i + 1) * step], src[i * step:(i + 1) * step])

    with ThreadPoolExecutor(nthreads) as ex:
        list(ex.map(part, range(nthreads)))
    return out


class DataArray:
    """``.data`` holder standing in for an xarray DataArray."""

    def __init__(self, data):
        self.data = data

    @property
    def shape(self):
        return self.data.shape

    @property
    def values(self):
        return self.data


class _WcsCore:
    def __init__(self, ctype, crpix, cdelt, crval):
        self.ctype = list(ctype)
        self.crpix = numpy.asarray(crpix, dtype=numpy.float64)
        self.cdelt = numpy.asarray(cdelt, dtype=numpy.float64)
        self.crval = numpy.asarray(crval, dtype=numpy.float64)


class WCS:
    """Linear 4-axis WCS (RA---SIN, DEC--SIN, STOKES, FREQ) as RASCIL images
    carry; ``sub([4]).wcs_world2pix`` gives the frequency channel index."""

    def __init__(self, ctype, crpix, cdelt, crval):
        self.wcs = _WcsCore(ctype, crpix, cdelt, crval)

    def sub(self, axes):
        idx = [a - 1 for a in axes]
        w = self.wcs
        return WCS([w.ctype[i] for i in idx], w.crpix[idx], w.cdelt[idx], w.crval[idx])

    def wcs_world2pix(self, *args):
        """Inverse of the linear transform; last argument is the origin."""
        origin = args[-1]
        world = args[:-1]
        w = self.wcs
        return [(numpy.asarray(x, dtype=numpy.float64) - w.crval[i]) / w.cdelt[i]
                + w.crpix[i] - 1 + origin for i, x in enumerate(world)]

    def deepcopy(self):
        return copy.deepcopy(self)


class _ImageAccessor:
    def __init__(self, im):
        self._im = im

    @property
    def wcs(self):
        return self._im._wcs

    @property
    def polarisation_frame(self):
        return self._im._polarisation_frame

    @property
    def phasecentre(self):
        return self._im._phasecentre

    @property
    def shape(self):
        return self._im["pixels"].data.shape

    @property
    def nchan(self):
        return self.shape[0]

    @property
    def npol(self):
        return self.shape[1]


class Image:
    """Image [nchan, npol, ny, nx] with a canonical 4-axis WCS."""

    def __init__(self, pixels, wcs, polarisation_frame, phasecentre):
        self._vars = {"pixels": DataArray(pixels)}
        self._wcs = wcs
        self._polarisation_frame = polarisation_frame
        self._phasecentre = phasecentre
        self.attrs = {}

    def __getitem__(self, key):
        return self._vars[key]

    @property
    def image_acc(self):
        return _ImageAccessor(self)

    def copy(self, deep=True, pixels=None):
        """Copy; ``deep`` copies the pixels (in parallel), ``pixels`` gives
        the copy a new pixel array instead."""
        if not deep and pixels is None:
            return copy.copy(self)
        new = copy.copy(self)
        new._wcs = copy.deepcopy(self._wcs)
        new.attrs = copy.deepcopy(self.attrs)
        data = self._vars["pixels"].data
        new._vars = {"pixels": DataArray(parallel_copy(data) if pixels is None else pixels)}
        return new


def create_image(npixel, cellsize, phasecentre, frequency=(1e8,), channel_bandwidth=(1e6,),
                 polarisation_frame=None, nchan=None, dtype=numpy.float64):
    """Canonical image like RASCIL's ``create_image``: RA---SIN/DEC--SIN with
    ``cdelt = (-cell, +cell)`` degrees and the phase centre at pixel
    ``npixel // 2`` (0-relative)."""
    polarisation_frame = polarisation_frame or PolarisationFrame("stokesI")
    frequency = numpy.atleast_1d(numpy.asarray(frequency, dtype=numpy.float64))
    channel_bandwidth = numpy.atleast_1d(numpy.asarray(channel_bandwidth, dtype=numpy.float64))
    nchan = nchan or len(frequency)
    df = channel_bandwidth[0] if nchan == 1 or len(frequency) < 2 else frequency[1] - frequency[0]
    cdeg = numpy.degrees(cellsize)
    wcs = WCS(["RA---SIN", "DEC--SIN", "STOKES", "FREQ"],
              [npixel // 2 + 1, npixel // 2 + 1, 1.0, 1.0],
              [-cdeg, cdeg, 1.0, df],
              [phasecentre.ra.deg, phasecentre.dec.deg, 1.0, frequency[0]])
    pixels = numpy.zeros((nchan, polarisation_frame.npol, npixel, npixel), dtype=dtype)
    return Image(pixels, wcs, polarisation_frame, phasecentre)


class _BVisAccessor:
    def __init__(self, bv):
        self._bv = bv

    @property
    def flagged_vis(self):
        """vis * (1 - flags) (``memory_data_models.py:1502-1507``)."""
        return self._bv["vis"].data * (1 - self._bv["flags"].data)

    @property
    def flagged_imaging_weight(self):
        """imaging_weight * (1 - flags) (``memory_data_models.py:1518-1523``)."""
        return self._bv["imaging_weight"].data * (1 - self._bv["flags"].data)

    @property
    def flagged_weight(self):
        return self._bv["weight"].data * (1 - self._bv["flags"].data)

    @property
    def polarisation_frame(self):
        return self._bv._polarisation_frame

    @property
    def uvw_lambda(self):
        f = self._bv.frequency.data / SPEED_OF_LIGHT
        return self._bv.uvw.data[..., numpy.newaxis, :] * f[:, numpy.newaxis]

    @property
    def nvis(self):
        return int(numpy.prod(self._bv["vis"].data.shape))


class BlockVisibility:
    """Visibilities [ntimes, nbaselines, nchan, npol] with uvw [ntimes, nbaselines, 3]."""

    def __init__(self, vis, uvw, frequency, phasecentre, polarisation_frame, flags=None,
                 weight=None, imaging_weight=None, time=None, baselines=None,
                 channel_bandwidth=None):
        vis = numpy.asarray(vis)
        self._vars = {
            "vis": DataArray(vis),
            "uvw": DataArray(numpy.asarray(uvw, dtype=numpy.float64)),
            "frequency": DataArray(numpy.asarray(frequency, dtype=numpy.float64)),
            "flags": DataArray(numpy.zeros(vis.shape, dtype=numpy.int64)
                               if flags is None else flags),
            "weight": DataArray(numpy.ones(vis.shape, dtype=numpy.float64)
                                if weight is None else weight),
            "imaging_weight": DataArray(numpy.ones(vis.shape, dtype=numpy.float64)
                                        if imaging_weight is None else imaging_weight),
        }
        self._polarisation_frame = polarisation_frame
        self.attrs = {"phasecentre": phasecentre, "polarisation_frame": polarisation_frame}
        self.time = DataArray(numpy.arange(vis.shape[0], dtype=numpy.float64)
                              if time is None else time)
        self.baselines = baselines
        self.channel_bandwidth = DataArray(
            numpy.ones(len(frequency)) * 1e6 if channel_bandwidth is None else channel_bandwidth)

    def __getitem__(self, key):
        return self._vars[key]

    def __getattr__(self, name):
        v = self.__dict__.get("_vars")
        if v is not None and name in v:
            return v[name]
        raise AttributeError(name)

    @property
    def phasecentre(self):
        return self.attrs["phasecentre"]

    @property
    def blockvisibility_acc(self):
        return _BVisAccessor(self)


def copy_visibility(bvis, zero=False, vis=None, skip_vis=False):
    """Deep copy, optionally zeroing vis (``visibility/base.py:105-118``).
    The arrays are copied in parallel; ``vis`` (same shape) becomes the
    copy's visibilities instead of a copy or zeros (predict writes the whole
    array, so copying or zeroing it first would be wasted).  ``skip_vis``
    leaves the copy's vis unset (``None``) for the caller to fill."""
    if not isinstance(bvis, BlockVisibility):
        new = copy.deepcopy(bvis)
        if vis is not None:
            new["vis"].data = vis
        elif zero:
            new["vis"].data[...] = 0.0
        return new
    new = copy.copy(bvis)
    new.__dict__ = {k: copy.deepcopy(v) for k, v in bvis.__dict__.items() if k != "_vars"}
    new._vars = {}
    copied = {}  # arrays shared inside the input stay shared in the copy (as deepcopy)
    for key, arr in bvis._vars.items():
        if key == "vis" and skip_vis:
            new._vars[key] = DataArray(None)
        elif key == "vis" and vis is not None:
            assert vis.shape == arr.data.shape
            new._vars[key] = DataArray(vis)
        elif key == "vis" and zero:
            new._vars[key] = DataArray(numpy.zeros_like(arr.data))
        else:
            if id(arr.data) not in copied:
                copied[id(arr.data)] = parallel_copy(arr.data)
            new._vars[key] = DataArray(copied[id(arr.data)])
    return new
