"""Seeded small problems shared by the tests."""
import numpy

from oracle.dft import SPEED_OF_LIGHT


def random_problem(seed=0, nrow=400, nchan=3, npix=64, pixsize=2e-3, wscale=800.0,
                   uvscale=3000.0, npol=1):
    rng = numpy.random.default_rng(seed)
    uvw = rng.uniform(-1, 1, (nrow, 3)) * numpy.array([uvscale, uvscale, wscale])
    freq = numpy.linspace(1.0e8, 1.4e8, nchan)
    shape = (nrow, nchan, npol)
    ms = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    wgt = rng.uniform(0.5, 1.0, shape)
    img = rng.normal(size=(npol, npix, npix))
    return dict(uvw=uvw, freq=freq, ms=ms, wgt=wgt, img=img, npix=npix, pixsize=pixsize)


def rel_rms(a, b):
    a = numpy.asarray(a)
    b = numpy.asarray(b)
    return float(numpy.linalg.norm((a - b).ravel()) / numpy.linalg.norm(b.ravel()))
