"""CPU restatement of RASCIL's imaging weights (test infrastructure only).

Follows ``rascil/processing_components/imaging/weighting.py:27-48``
(``weight_visibility``) and ``griddata/gridding.py``:

* ``create_griddata_from_image`` (``griddata/operations.py:71-107``): an
  image-sized uv grid, ``cdelt_u = 1 / (nx cdelt_x d2r)``, ``cdelt_v = 1 /
  (ny cdelt_y d2r)`` (image cdelt in degrees, RA negative), reference pixel
  ``(nx // 2, ny // 2)`` (0-based), reference value 0;
* ``spatial_mapping`` (``gridding.py:68-175``, no convolution function): the
  cell of a sample is ``round((u - 0) / cdelt_u + crpix - 1)`` (numpy round,
  half to even) with u in wavelengths (``uvw * f / c``, nan -> 0); a cell
  outside the grid is an error (RASCIL asserts);
* ``grid_blockvisibility_weight_to_griddata`` (``gridding.py:260-306``): the
  grid accumulates the flagged imaging weights, channel by channel, pol by
  pol, row by row, and sumwt per (image channel, pol) in the same order;
* ``griddata_blockvisibility_reweight`` (``gridding.py:332-425``): uniform
  ``w <- w (w / G)``; robust ``w <- w ((1 + f2 w) / (1 + f2 G))`` with
  ``f2 = (5 10^-R)^2 sum(w) / sum(G^2)``; both 0 where ``G <= 0``; natural
  ``imaging_weight <- weight``.

Used only by the tests as the checker of ``rascil_gb300.imaging.weighting``.
"""
import numpy

SPEED_OF_LIGHT = 299792458.0


def uv_cells(uvw, freq, nx, ny, cdelt_x_deg, cdelt_y_deg):
    """(pu, pv) int arrays [nrows, nchan] of each sample's grid cell."""
    d2r = numpy.pi / 180.0
    cdu = 1.0 / (nx * cdelt_x_deg * d2r)
    cdv = 1.0 / (ny * cdelt_y_deg * d2r)
    k = numpy.asarray(freq, dtype=numpy.float64) / SPEED_OF_LIGHT
    uvw = numpy.asarray(uvw, dtype=numpy.float64).reshape(-1, 3)
    u = numpy.nan_to_num(uvw[:, 0:1] * k[None, :])
    v = numpy.nan_to_num(uvw[:, 1:2] * k[None, :])
    pu = numpy.round((u - 0.0) / cdu + float(nx // 2 + 1) - 1.0).astype(numpy.int64)
    pv = numpy.round((v - 0.0) / cdv + float(ny // 2 + 1) - 1.0).astype(numpy.int64)
    return pu, pv


def weight_grid(pu, pv, fimw, vis_to_im, nchan_img, nx, ny):
    """Gridded flagged imaging weights [nchan_img, npol, ny, nx] and sumwt,
    accumulated in the reference's order."""
    nrows, nchan, npol = fimw.shape
    if (pu.min() < 0 or pu.max() >= nx or pv.min() < 0 or pv.max() >= ny):
        raise ValueError("a sample's uv cell lies outside the weighting grid")
    grid = numpy.zeros((nchan_img, npol, ny, nx))
    sumwt = numpy.zeros((nchan_img, npol))
    for c in range(nchan):
        ic = vis_to_im[c]
        for p in range(npol):
            numpy.add.at(grid[ic, p], (pv[:, c], pu[:, c]), fimw[:, c, p])
            sumwt[ic, p] = numpy.cumsum(numpy.concatenate([[sumwt[ic, p]], fimw[:, c, p]]))[-1]
    return grid, sumwt


def reweight(grid, pu, pv, fimw, weight, vis_to_im, scheme, robustness=0.0):
    """New imaging weights [nrows, nchan, npol] (flags applied through fimw)."""
    nrows, nchan, npol = fimw.shape
    if scheme == "natural":
        return numpy.array(weight, dtype=numpy.float64, copy=True)
    out = numpy.array(fimw, dtype=numpy.float64, copy=True)
    if scheme == "robust":
        sumlocwt = numpy.sum(grid ** 2)
        sumwt = numpy.sum(fimw)
        f2 = (5.0 * numpy.power(10.0, -robustness)) ** 2 * sumwt / sumlocwt
    elif scheme != "uniform":
        raise ValueError("weighting %s not supported" % scheme)
    for p in range(npol):
        for c in range(nchan):
            g = grid[vis_to_im[c], p, pv[:, c], pu[:, c]]
            x = out[:, c, p]
            pos = g > 0.0
            if scheme == "uniform":
                x[pos] *= x[pos] / g[pos]
            else:
                x[pos] *= (1 + f2 * x[pos]) / (1 + f2 * g[pos])
            x[~pos] = 0.0
    return out


def weight_visibility(uvw, freq, weight, imaging_weight, flags, vis_to_im, nchan_img, nx, ny,
                      cdelt_x_deg, cdelt_y_deg, scheme="uniform", robustness=0.0):
    """Whole operation on [nrows, nchan, npol] arrays: returns (new imaging
    weights, grid, sumwt)."""
    pu, pv = uv_cells(uvw, freq, nx, ny, cdelt_x_deg, cdelt_y_deg)
    fimw = numpy.asarray(imaging_weight, dtype=numpy.float64) * (1 - numpy.asarray(flags))
    grid, sumwt = weight_grid(pu, pv, fimw, vis_to_im, nchan_img, nx, ny)
    return reweight(grid, pu, pv, fimw, weight, vis_to_im, scheme, robustness), grid, sumwt
