"""ctypes driver of ``oracle/wgridder.c``: the FP64 multithreaded CPU
w-stacking gridder (oracle / timed CPU baseline; test infrastructure only).

Planning and per-item coordinates come from :mod:`oracle.wgridder`; the
per-plane gridding, degridding and w-screens run in C with OpenMP; the
2-D FFTs use ``scipy.fft`` (pocketfft) with all worker threads.  Like
RASCIL's ng path (``rascil/processing_components/imaging/ng.py:227-277``),
each call handles one polarisation.

``planes`` restricts a call to a subset of w-planes; the benchmark uses
an evenly spread subset as a bounded sample and scales the time by
``nplanes / len(planes)``.
"""
import ctypes
import os
import subprocess
import time

import numpy
import scipy.fft

from . import wgridder as owg
from .dft import SPEED_OF_LIGHT

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "wgridder.c")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libogridder.so")
_lib = None


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", SRC, "-o",
           LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        i32, i64, dbl, vp = ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
        lib.og_grid_plane.argtypes = [i32, i32, i32, dbl, i32, i32] + [vp] * 7 + [vp, vp, i32,
                                                                                  vp, i32]
        lib.og_degrid_plane.argtypes = [i32, i32, i32, dbl, i32, i32] + [vp] * 6 + [vp, i64, vp,
                                                                                    vp, i32]
        lib.og_screen_acc.argtypes = [i32, i32, i32, i32, i32, dbl, vp, vp, vp, i32]
        lib.og_screen_pad.argtypes = [i32, i32, i32, i32, i32, dbl, vp, vp, vp, i32]
        lib.og_max_threads.restype = i32
        _lib = lib
    return _lib


def max_threads():
    return int(_load().og_max_threads())


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Prepared:
    """Per-item coordinates for a plan (items = (row, channel) pairs, or any
    subset of them given directly in wavelengths)."""

    def __init__(self, plan, u, v, w):
        self.plan = plan
        p0, q0, k0, du, dv, dwf, ph, flip = plan.coords_lambda(u, v, w)
        self.flip = flip  # mirrored items: grid conj(value), predict the conjugate
        self.p0 = numpy.ascontiguousarray(p0, dtype=numpy.int32)
        self.q0 = numpy.ascontiguousarray(q0, dtype=numpy.int32)
        self.k0 = numpy.ascontiguousarray(k0, dtype=numpy.int32)
        self.du = numpy.ascontiguousarray(du)
        self.dv = numpy.ascontiguousarray(dv)
        self.dwf = numpy.ascontiguousarray(dwf)
        self.ph = ph
        self.by_k0 = numpy.argsort(self.k0, kind="stable")
        self.k0_sorted = self.k0[self.by_k0]
        pl = self.plan
        if pl.do_w:
            t = pl.pixel_t().T  # [ny][nx]
            self.tprime = numpy.ascontiguousarray(t - pl.tc)
        else:
            self.tprime = None
        self.corr = numpy.ascontiguousarray(pl.correction().T)  # [ny][nx]
        # bands of equal height h >= max(W, 8) dividing the grid into an even
        # number of them: an item's support then reaches only its own band and
        # the next, and the last band (odd) wraps into band 0 (even), so the
        # two parity passes never write one row from two threads (a shorter
        # last band would let the band before it wrap into band 0 as well)
        h = max(pl.W, 8)
        while pl.ngy % h or (pl.ngy // h) % 2:
            h += 1
        self.band_h = h
        self.nbands = pl.ngy // h

    @classmethod
    def from_uvw(cls, uvw, freq, nx, ny, dx, dy, epsilon, do_w, sigma=2.0):
        s = numpy.asarray(freq, dtype=numpy.float64) / SPEED_OF_LIGHT
        u = (uvw[:, 0:1] * s).ravel()
        v = (uvw[:, 1:2] * s).ravel()
        w = (uvw[:, 2:3] * s).ravel()
        plan = owg.Plan(nx, ny, dx, dy, epsilon, do_w, *owg.w_range(w, do_w), sigma)
        return cls(plan, u, v, w)

    def items_of_plane(self, k):
        W = self.plan.W if self.plan.do_w else 1
        lo = numpy.searchsorted(self.k0_sorted, k - W + 1, side="left")
        hi = numpy.searchsorted(self.k0_sorted, k, side="right")
        return self.by_k0[lo:hi]

    def banded(self, idx):
        band = self.q0[idx] // self.band_h
        order = numpy.argsort(band, kind="stable")
        idx = numpy.ascontiguousarray(idx[order], dtype=numpy.int64)
        starts = numpy.searchsorted(band[order], numpy.arange(self.nbands + 1)).astype(numpy.int64)
        return idx, numpy.ascontiguousarray(starts)


def _tick(timing, key, t0, n=0):
    """Add the seconds since t0 (and n item-planes) to timing[key]."""
    if timing is not None:
        timing[key] = timing.get(key, 0.0) + time.perf_counter() - t0
        timing["item_planes"] = timing.get("item_planes", 0) + n
    return time.perf_counter()


def grid_items(pr, c, nthreads=None, planes=None, timing=None):
    """Dirty image [ny][nx] from item values c (weights applied), FP64.
    ``timing`` (a dict), when given, accumulates the seconds spent on the
    items' spreading ("items") and on the per-plane transforms and screens
    ("planes"), and the item-planes spread ("item_planes")."""
    lib = _load()
    nthreads = nthreads or max_threads()
    pl = pr.plan
    c = numpy.asarray(c, dtype=numpy.complex128).ravel()
    c = numpy.ascontiguousarray(numpy.where(pr.flip, numpy.conj(c), c) * pr.ph)
    cv = c.view(numpy.float64)
    acc = numpy.zeros((pl.ny, pl.nx))
    grid = numpy.zeros((pl.ngy, pl.ngx), dtype=numpy.complex128)
    for k in (range(pl.nplanes) if planes is None else planes):
        idx = pr.items_of_plane(k)
        if idx.size == 0:
            continue
        t0 = time.perf_counter()
        order, starts = pr.banded(idx)
        grid[...] = 0
        lib.og_grid_plane(pl.ngx, pl.ngy, pl.W, pl.beta, int(pl.do_w), int(k), _p(pr.p0),
                          _p(pr.q0), _p(pr.k0), _p(pr.du), _p(pr.dv), _p(pr.dwf), _p(cv),
                          _p(order), _p(starts), int(pr.nbands), _p(grid.view(numpy.float64)),
                          nthreads)
        t0 = _tick(timing, "items", t0, idx.size)
        img = scipy.fft.ifft2(grid, norm="forward", workers=nthreads, overwrite_x=True)
        img = numpy.ascontiguousarray(img)
        lib.og_screen_acc(pl.nx, pl.ny, pl.ngx, pl.ngy, int(pl.do_w), float(pl.w_plane(k)),
                          None if pr.tprime is None else _p(pr.tprime),
                          _p(img.view(numpy.float64)), _p(acc), nthreads)
        _tick(timing, "planes", t0)
    return acc * pr.corr


def degrid_items(pr, image_yx, nthreads=None, planes=None, timing=None):
    """Item values from a real image [ny][nx], FP64 (``timing`` as in
    :func:`grid_items`)."""
    lib = _load()
    nthreads = nthreads or max_threads()
    pl = pr.plan
    img = numpy.ascontiguousarray(numpy.asarray(image_yx, dtype=numpy.float64) * pr.corr)
    out = numpy.zeros(pr.p0.size, dtype=numpy.complex128)
    ov = out.view(numpy.float64)
    grid = numpy.zeros((pl.ngy, pl.ngx), dtype=numpy.complex128)
    for k in (range(pl.nplanes) if planes is None else planes):
        idx = pr.items_of_plane(k)
        if idx.size == 0:
            continue
        t0 = time.perf_counter()
        lib.og_screen_pad(pl.nx, pl.ny, pl.ngx, pl.ngy, int(pl.do_w), float(pl.w_plane(k)),
                          None if pr.tprime is None else _p(pr.tprime), _p(img),
                          _p(grid.view(numpy.float64)), nthreads)
        g = numpy.ascontiguousarray(scipy.fft.fft2(grid, workers=nthreads))
        t0 = _tick(timing, "planes", t0)
        idx = numpy.ascontiguousarray(idx, dtype=numpy.int64)
        lib.og_degrid_plane(pl.ngx, pl.ngy, pl.W, pl.beta, int(pl.do_w), int(k), _p(pr.p0),
                            _p(pr.q0), _p(pr.k0), _p(pr.du), _p(pr.dv), _p(pr.dwf), _p(idx),
                            int(idx.size), _p(g.view(numpy.float64)), _p(ov), nthreads)
        _tick(timing, "items", t0, idx.size)
    out = out * numpy.conj(pr.ph)
    return numpy.where(pr.flip, numpy.conj(out), out)


def ms2dirty(uvw, freq, ms, wgt, npix_x, npix_y, pixsize_x, pixsize_y, epsilon, do_wstacking,
             nthreads=None, planes=None, sigma=2.0):
    """Dirty image [npix_x, npix_y] (ducc0 convention), FP64, on the CPU."""
    pr = Prepared.from_uvw(uvw, freq, npix_x, npix_y, pixsize_x, pixsize_y, epsilon,
                           do_wstacking, sigma)
    c = numpy.asarray(ms, dtype=numpy.complex128)
    if wgt is not None:
        c = c * numpy.asarray(wgt, dtype=numpy.float64)
    return grid_items(pr, c, nthreads, planes).T


def dirty2ms(uvw, freq, dirty, wgt, pixsize_x, pixsize_y, epsilon, do_wstacking,
             nthreads=None, planes=None, sigma=2.0):
    """Visibilities [nrow, nchan] (ducc0 convention), FP64, on the CPU."""
    npix_x, npix_y = dirty.shape
    pr = Prepared.from_uvw(uvw, freq, npix_x, npix_y, pixsize_x, pixsize_y, epsilon,
                           do_wstacking, sigma)
    out = degrid_items(pr, numpy.asarray(dirty).T, nthreads, planes)
    out = out.reshape(uvw.shape[0], len(freq))
    if wgt is not None:
        out = out * wgt
    return out
