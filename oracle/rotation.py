"""CPU restatement of RASCIL's tangent-plane phase rotation (test
infrastructure only: the checker of ``gb_phase_rotate`` and of the phase
shift fused into the gridder plans).

Follows ``rascil/processing_components/visibility/base.py``:

* ``calculate_blockvisibility_phasor`` (``:1248-1264``): with
  ``s = (l, m, sqrt(1 - l^2 - m^2) - 1)`` of the new phase centre about the
  old one, ``phasor = exp(-2 pi i uvw_lambda . s)`` for every (row,
  channel), the same for every pol;
* ``phaserotate_visibility`` (``:296-357``): nothing when ``|n - 1| <
  1e-15``; otherwise vis times ``conj(phasor)``, or times ``phasor`` when
  ``inverse``; ``tangent=False`` also rotates uvw through the XYZ frame
  (``uvw_to_xyz`` at the old centre, ``xyz_to_uvw`` at the new, with
  hour angle = -ra).

Pinned against ``tests/golden/rotation.npz`` (made by running the
reference's own functions, ``tests/golden/make_golden.py``).
"""
import numpy

SPEED_OF_LIGHT = 299792458.0


def direction(l, m):
    """s = (l, m, sqrt(1 - l^2 - m^2) - 1)."""
    return numpy.array([l, m, numpy.sqrt(1.0 - l * l - m * m) - 1.0])


def phasor(uvw, freq, s):
    """exp(-2 pi i uvw_lambda . s), [..., nchan] for uvw [..., 3] (metres)."""
    uvw_lambda = numpy.asarray(uvw)[..., None, :] * (numpy.asarray(freq) / SPEED_OF_LIGHT)[:, None]
    return numpy.exp(-2j * numpy.pi * (uvw_lambda @ numpy.asarray(s)))


def simulate_point(dist_uvw, l, m):
    """exp(-2 pi i dist_uvw . s) (``util/coordinate_support.py:526-538``),
    dist_uvw in wavelengths."""
    return numpy.exp(-2j * numpy.pi * (numpy.asarray(dist_uvw) @ direction(l, m)))


def phaserotate(vis, uvw, freq, lmn, inverse=False):
    """vis [..., nchan, npol] rotated by the phasor of lmn = (l, m, n - 1)."""
    if abs(lmn[2]) < 1e-15:
        return vis
    ph = phasor(uvw, freq, direction(lmn[0], lmn[1]))[..., None]
    return vis * (ph if inverse else numpy.conj(ph))


def uvw_to_xyz(uvw, ha, dec):
    u, v, w = uvw[..., 0], uvw[..., 1], uvw[..., 2]
    v0 = v * numpy.sin(dec) - w * numpy.cos(dec)
    z = v * numpy.cos(dec) + w * numpy.sin(dec)
    x = u * numpy.cos(ha) + v0 * numpy.sin(ha)
    y = -u * numpy.sin(ha) + v0 * numpy.cos(ha)
    return numpy.stack([x, y, z], axis=-1)


def xyz_to_uvw(xyz, ha, dec):
    x, y, z = xyz[..., 0], xyz[..., 1], xyz[..., 2]
    u = x * numpy.cos(ha) - y * numpy.sin(ha)
    v0 = x * numpy.sin(ha) + y * numpy.cos(ha)
    w = z * numpy.sin(dec) - v0 * numpy.cos(dec)
    v = z * numpy.cos(dec) + v0 * numpy.sin(dec)
    return numpy.stack([u, v, w], axis=-1)


def rotate_uvw(uvw, old_ra, old_dec, new_ra, new_dec):
    return xyz_to_uvw(uvw_to_xyz(uvw, -old_ra, old_dec), -new_ra, new_dec)
