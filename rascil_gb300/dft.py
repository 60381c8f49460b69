"""GPU direct Fourier transforms (component DFT and exact dirty pixels).

:func:`dft_components` is the GPU form of the reference's
``dft_skycomponent_visibility`` kernel (``rascil/processing_components/
imaging/dft.py:44-62,123-178``; CUDA source ``:181-258``);
:func:`dft_pixels` evaluates the exact direct sum that the gridder
approximates at chosen pixels (ducc0 ms2dirty convention), the truth used
for accuracy reports at sizes no CPU oracle reaches.
"""
import ctypes

import numpy
import torch

from . import _lib
from .wgridder import _ptr, _stream


def dft_components(uvw, freq, lmn, flux, precision="fp64", exact=True):
    """vis [nrows, nchan, npol] from components.

    :param uvw: [nrows, 3] float64 CUDA tensor (metres)
    :param freq: [nchan] float64 CUDA tensor (Hz)
    :param lmn: [ncomp, 3] float64 (l, m, n-1)
    :param flux: [ncomp, nchan, npol] complex128
    """
    lib = _lib.load()
    nrows, nchan = int(uvw.shape[0]), int(freq.shape[0])
    dev = uvw.device
    lmn = torch.as_tensor(lmn, dtype=torch.float64).to(dev).contiguous()
    flux = torch.as_tensor(flux).to(dev, torch.complex128).contiguous()
    ncomp, _, npol = flux.shape
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    vis = torch.empty((nrows, nchan, npol), dtype=cdt, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.gb_dft_components(_ptr(uvw), _ptr(freq), nrows, nchan, _ptr(lmn),
                                         _ptr(flux), int(ncomp), int(npol), _ptr(vis),
                                         _lib.GB_FP64 if precision == "fp64" else _lib.GB_FP32,
                                         1 if exact else 0, _stream(dev)), "gb_dft_components")
    return vis


def dft_pixels(uvw, freq, ms, wgt, pixels, npix_x, npix_y, pixsize_x, pixsize_y,
               do_wstacking, pol=0, exact=True):
    """Exact ms2dirty values (ducc0 convention) at ``pixels`` [n, 2] (ix, iy).

    :param ms: [nrows, nchan, npol] complex CUDA tensor
    :param wgt: same shape real tensor (same precision) or None
    """
    lib = _lib.load()
    dev = uvw.device
    nrows, nchan = int(uvw.shape[0]), int(freq.shape[0])
    npol = int(ms.shape[-1]) if ms.dim() == 3 else 1
    prec = _lib.GB_FP64 if ms.dtype == torch.complex128 else _lib.GB_FP32
    pix = torch.as_tensor(numpy.asarray(pixels, dtype=numpy.int32)).to(dev).contiguous()
    out = torch.empty(pix.shape[0], dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.gb_dft_pixels(_ptr(uvw), _ptr(freq), nrows, nchan, npol, int(pol),
                                     _ptr(ms.contiguous()), prec,
                                     None if wgt is None else _ptr(wgt.contiguous()), _ptr(pix),
                                     int(pix.shape[0]), int(npix_x), int(npix_y),
                                     float(pixsize_x), float(pixsize_y),
                                     1 if do_wstacking else 0, 1 if exact else 0, _ptr(out),
                                     _stream(dev)), "gb_dft_pixels")
    return out
