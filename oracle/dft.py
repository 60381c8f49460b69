"""FP64 direct Fourier transforms (oracle; test infrastructure only).

* :func:`dft_cpu_looped` restates the reference's component DFT,
  ``rascil/processing_components/imaging/dft.py:261-281``:
  ``V[t,b,f,p] = sum_c flux[c,f,p] * exp(-2 pi i uvw_lambda[t,b,f] . dir[c])``
  with ``dir = (l, m, n - 1)``.
* :func:`ms2dirty_dft` / :func:`dirty2ms_dft` are the exact operators that
  ``ducc0.wgridder.ms2dirty`` / ``dirty2ms`` approximate, in ducc0's
  argument convention (the flipped u and w that ``ng.py:73-77,201-204``
  pass, image axis 0 = x).  With ``x = (i - nx/2) dx``, ``y = (j - ny/2) dy``,
  ``nm1 = n - 1 = -(x^2+y^2)/(1+sqrt(1-x^2-y^2))`` (0 without w-stacking)::

      dirty[i,j] = sum_{r,c} Re(wgt ms exp(+2 pi i f_c/c (x u + y v - w nm1))) / n
      ms[r,c]    = wgt sum_{i,j} dirty[i,j] / n exp(-2 pi i f_c/c (x u + y v - w nm1))

  The two are adjoint to each other (real inner product on images,
  Re of the complex one on visibilities).
"""

import numpy

SPEED_OF_LIGHT = 299792458.0  # rascil/phyconst.py:6


def dft_cpu_looped(direction_cosines, uvw_lambda, vfluxes):
    """Component DFT, restating ``imaging/dft.py:261-281``.

    :param direction_cosines: [ncomp, 3] rows (l, m, n-1)
    :param uvw_lambda: [ntimes, nbaselines, nchan, 3] uvw in wavelengths
    :param vfluxes: [ncomp, nchan, npol] complex fluxes
    :return: [ntimes, nbaselines, nchan, npol] complex128
    """
    ncomp = direction_cosines.shape[0]
    ntimes, nbaselines, nchan, _ = uvw_lambda.shape
    npol = vfluxes.shape[-1]
    vis = numpy.zeros([ntimes, nbaselines, nchan, npol], dtype=numpy.complex128)
    for icomp in range(ncomp):
        phase = numpy.einsum("tbfs,s->tbf", uvw_lambda, direction_cosines[icomp])
        phasor = numpy.exp(-2j * numpy.pi * phase)
        for pol in range(npol):
            vis[..., pol] += vfluxes[icomp, :, pol] * phasor
    return vis


def _pixel_coords(npix_x, npix_y, pixsize_x, pixsize_y, do_wstacking):
    x = (numpy.arange(npix_x) - npix_x // 2) * pixsize_x
    y = (numpy.arange(npix_y) - npix_y // 2) * pixsize_y
    xx, yy = numpy.meshgrid(x, y, indexing="ij")
    r2 = xx * xx + yy * yy
    if do_wstacking:
        nm1 = -r2 / (numpy.sqrt(1.0 - r2) + 1.0)
    else:
        nm1 = numpy.zeros_like(r2)
    return xx, yy, nm1


def ms2dirty_dft(uvw, freq, ms, wgt, npix_x, npix_y, pixsize_x, pixsize_y,
                 do_wstacking, pixel_subset=None, chunk=256):
    """Exact (direct-sum) dirty image in ducc0's convention.

    :param uvw: [nrow, 3] metres (already u/w-flipped by the caller as ng.py does)
    :param freq: [nchan] Hz
    :param ms: [nrow, nchan] complex
    :param wgt: [nrow, nchan] real or None
    :param pixel_subset: optional (ix, iy) integer arrays; returns only those pixels
    :return: [npix_x, npix_y] float64, or [len(ix)] for a subset
    """
    xx, yy, nm1 = _pixel_coords(npix_x, npix_y, pixsize_x, pixsize_y, do_wstacking)
    if pixel_subset is not None:
        ix, iy = pixel_subset
        xx, yy, nm1 = xx[ix, iy], yy[ix, iy], nm1[ix, iy]
    shape = xx.shape
    xs, ys, ns = xx.ravel(), yy.ravel(), nm1.ravel()
    vals = numpy.asarray(ms, dtype=numpy.complex128)
    if wgt is not None:
        vals = vals * wgt
    scale = numpy.asarray(freq, dtype=numpy.float64) / SPEED_OF_LIGHT
    u = (uvw[:, 0:1] * scale).ravel()
    v = (uvw[:, 1:2] * scale).ravel()
    w = (uvw[:, 2:3] * scale).ravel()
    c = vals.ravel()
    out = numpy.zeros(xs.size)
    for s in range(0, xs.size, chunk):
        ph = (numpy.outer(xs[s:s + chunk], u) + numpy.outer(ys[s:s + chunk], v)
              - numpy.outer(ns[s:s + chunk], w))
        out[s:s + chunk] = (numpy.exp(2j * numpy.pi * ph) @ c).real
    out = out / (ns + 1.0)
    return out.reshape(shape)


def dirty2ms_dft(uvw, freq, dirty, wgt, pixsize_x, pixsize_y, do_wstacking,
                 row_subset=None, chunk=64):
    """Exact (direct-sum) visibilities in ducc0's convention.

    :param dirty: [npix_x, npix_y] real
    :param row_subset: optional row indices; returns only those rows
    :return: [nrow, nchan] complex128
    """
    npix_x, npix_y = dirty.shape
    xx, yy, nm1 = _pixel_coords(npix_x, npix_y, pixsize_x, pixsize_y, do_wstacking)
    nz = dirty != 0
    img = (dirty[nz] / (nm1[nz] + 1.0)).astype(numpy.complex128)
    xs, ys, ns = xx[nz], yy[nz], nm1[nz]
    if row_subset is not None:
        uvw = uvw[row_subset]
        if wgt is not None:
            wgt = wgt[row_subset]
    scale = numpy.asarray(freq, dtype=numpy.float64) / SPEED_OF_LIGHT
    nrow, nchan = uvw.shape[0], scale.size
    out = numpy.zeros((nrow, nchan), dtype=numpy.complex128)
    for ch in range(nchan):
        u = uvw[:, 0] * scale[ch]
        v = uvw[:, 1] * scale[ch]
        w = uvw[:, 2] * scale[ch]
        for s in range(0, nrow, chunk):
            ph = (numpy.outer(u[s:s + chunk], xs) + numpy.outer(v[s:s + chunk], ys)
                  - numpy.outer(w[s:s + chunk], ns))
            out[s:s + chunk, ch] = numpy.exp(-2j * numpy.pi * ph) @ img
    if wgt is not None:
        out = out * wgt
    return out


def lmn_of_direction(ra, dec, ra0, dec0):
    """Direction cosines of (ra, dec) about the phase centre (ra0, dec0).

    Same quantity as ``skycoord_to_lmn``
    (``rascil/processing_components/util/coordinate_support.py:446-465``):
    l east-wards, m north-wards, n towards the source; returns (l, m, n-1).
    """
    dra = ra - ra0
    l = numpy.cos(dec) * numpy.sin(dra)
    m = numpy.sin(dec) * numpy.cos(dec0) - numpy.cos(dec) * numpy.sin(dec0) * numpy.cos(dra)
    n = numpy.sin(dec) * numpy.sin(dec0) + numpy.cos(dec) * numpy.cos(dec0) * numpy.cos(dra)
    return l, m, n - 1.0
