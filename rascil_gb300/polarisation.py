"""Polarisation frames and frame conversion as small complex matrices.

Same frames, product order and conversions as
``rascil/data_models/polarisation.py`` (frames ``:88-106``, conversions
``:220-419``).  Each supported conversion is expressed as one
[npol_out, npol_in] complex matrix, so the GPU kernels can fuse it into the
visibility pre-pass of invert and the epilogue of predict instead of
making a separate pass over the data.  The matrices are Thompson, Moran &
Swenson eq. 4.58 (linear) and 4.59 (circular) and their inverses.
"""

import numpy

_FRAMES = {
    "circular": ["RR", "RL", "LR", "LL"],
    "circularnp": ["RR", "LL"],
    "linear": ["XX", "XY", "YX", "YY"],
    "linearnp": ["XX", "YY"],
    "stokesIQUV": ["I", "Q", "U", "V"],
    "stokesIV": ["I", "V"],
    "stokesIQ": ["I", "Q"],
    "stokesI": ["I"],
}


class PolarisationFrame:
    """Polarisation frame after correlation (stokesI, stokesIQUV, linear, ...)."""

    polarisation_frames = {k: {n: i for i, n in enumerate(v)} for k, v in _FRAMES.items()}

    def __init__(self, name):
        if name not in _FRAMES:
            raise ValueError("Unknown polarisation frame %s" % str(name))
        self.type = name
        self.translations = self.polarisation_frames[name]

    def __eq__(self, other):
        if other is None:
            return False
        return self.type == getattr(other, "type", other)

    def __hash__(self):
        return hash(self.type)

    def __str__(self):
        return self.type

    __repr__ = __str__

    @property
    def npol(self):
        return len(_FRAMES[self.type])

    @property
    def names(self):
        return list(_FRAMES[self.type])


# Stokes -> correlation products (TMS 4.58 / 4.59)
_STOKES_TO_LINEAR = numpy.array([[1, 1, 0, 0], [0, 0, 1, 1j], [0, 0, 1, -1j], [1, -1, 0, 0]],
                                dtype=numpy.complex128)
_STOKES_TO_CIRCULAR = numpy.array([[1, 0, 0, 1], [0, -1j, 1, 0], [0, -1j, -1, 0], [1, 0, 0, -1]],
                                  dtype=numpy.complex128)
_STOKES2_TO_PAIR = numpy.array([[1, 1], [1, -1]], dtype=numpy.complex128)


def _name(f):
    return getattr(f, "type", f)


def conversion_matrix(ipf, opf):
    """[npol_out, npol_in] complex matrix taking frame ``ipf`` to ``opf``.

    Supports exactly the conversions of ``convert_pol_frame``
    (``rascil/data_models/polarisation.py:367-419``); raises ValueError
    otherwise.  Identity frames give the identity matrix.
    """
    a, b = _name(ipf), _name(opf)
    if a not in _FRAMES or b not in _FRAMES:
        raise ValueError("Unknown polarisation conversion: {} to {}".format(a, b))
    if a == b:
        return numpy.eye(len(_FRAMES[a]), dtype=numpy.complex128)
    pairs = {
        ("linear", "stokesIQUV"): numpy.linalg.inv(_STOKES_TO_LINEAR),
        ("circular", "stokesIQUV"): numpy.linalg.inv(_STOKES_TO_CIRCULAR),
        ("stokesIQUV", "linear"): _STOKES_TO_LINEAR,
        ("stokesIQUV", "circular"): _STOKES_TO_CIRCULAR,
        ("linearnp", "stokesIQ"): numpy.linalg.inv(_STOKES2_TO_PAIR),
        ("circularnp", "stokesIV"): numpy.linalg.inv(_STOKES2_TO_PAIR),
        ("stokesIQ", "linearnp"): _STOKES2_TO_PAIR,
        ("stokesIV", "circularnp"): _STOKES2_TO_PAIR,
        ("linear", "stokesI"): numpy.array([[0.5, 0, 0, 0.5]], dtype=numpy.complex128),
        ("circular", "stokesI"): numpy.array([[0.5, 0, 0, 0.5]], dtype=numpy.complex128),
        ("linearnp", "stokesI"): numpy.array([[0.5, 0.5]], dtype=numpy.complex128),
        ("circularnp", "stokesI"): numpy.array([[0.5, 0.5]], dtype=numpy.complex128),
        ("stokesIQUV", "stokesI"): numpy.array([[1, 0, 0, 0]], dtype=numpy.complex128),
        ("stokesI", "stokesIQUV"): numpy.array([[1], [0], [0], [0]], dtype=numpy.complex128),
    }
    if (a, b) not in pairs:
        raise ValueError("Unknown polarisation conversion: {} to {}".format(a, b))
    m = pairs[(a, b)]
    # the inverses above are exact in binary (entries 0, +-0.5, +-0.5j)
    return numpy.round(m.real * 4) / 4 + 1j * numpy.round(m.imag * 4) / 4


def convert_pol_frame(polvec, ipf, opf, polaxis=1):
    """Convert ``polvec`` from frame ``ipf`` to ``opf`` along ``polaxis``."""
    if _name(ipf) == _name(opf):
        return polvec
    m = conversion_matrix(ipf, opf)
    v = numpy.asarray(polvec)
    out = numpy.tensordot(m, v, axes=(1, polaxis))
    return numpy.moveaxis(out, 0, polaxis)
