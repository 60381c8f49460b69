"""Seeded synthetic interferometer observations in the shapes the
benchmarks name (no configuration files or datasets are needed).

Geometry restates the reference's: ENU -> celestial XYZ
(``rascil/processing_components/util/coordinate_support.py:213-226``,
``enu_to_xyz``), XYZ -> uvw for an hour angle and declination
(``:352-379``, ``xyz_to_uvw``), baselines ant2 - ant1 for ant1 < ant2
(``rascil/processing_components/visibility/base.py:246-258``), hour
angles in radians (``times_are_ha``).  Cross-correlations only.
"""
import numpy

from .data_models import BlockVisibility, SkyDirection, create_image
from .polarisation import PolarisationFrame, conversion_matrix

SPEED_OF_LIGHT = 299792458.0


def enu_to_xyz(e, n, u, lat):
    sl, cl = numpy.sin(lat), numpy.cos(lat)
    return -sl * n + cl * u, e, cl * n + sl * u


def xyz_to_uvw(xyz, ha, dec):
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    u = x * numpy.cos(ha) - y * numpy.sin(ha)
    v0 = x * numpy.sin(ha) + y * numpy.cos(ha)
    w = z * numpy.sin(dec) - v0 * numpy.cos(dec)
    v = z * numpy.cos(dec) + v0 * numpy.sin(dec)
    return numpy.stack([u, v, w], axis=-1)


def disk_positions(rng, n, radius):
    r = radius * numpy.sqrt(rng.uniform(0.0, 1.0, n))
    phi = rng.uniform(0.0, 2 * numpy.pi, n)
    return r * numpy.cos(phi), r * numpy.sin(phi)


def log_radial_positions(rng, n, rmin, rmax):
    r = numpy.exp(rng.uniform(numpy.log(rmin), numpy.log(rmax), n))
    phi = rng.uniform(0.0, 2 * numpy.pi, n)
    return r * numpy.cos(phi), r * numpy.sin(phi)


def baseline_uvw(east, north, lat, ha, dec):
    """uvw [ntimes, nbaselines, 3] (metres) for all ant1 < ant2 pairs."""
    x, y, z = enu_to_xyz(east, north, numpy.zeros_like(east), lat)
    xyz = numpy.stack([x, y, z], axis=-1)
    a1, a2 = numpy.triu_indices(len(east), k=1)
    out = numpy.empty((len(ha), len(a1), 3))
    for t, h in enumerate(ha):
        ant = xyz_to_uvw(xyz, h, dec)
        out[t] = ant[a2] - ant[a1]
    return out


def power_law_fluxes(rng, n, smin, smax, index):
    """Fluxes with dN/dS ~ S^-index between smin and smax (inverse CDF)."""
    a = 1.0 - index
    u = rng.uniform(0.0, 1.0, n)
    return (smin ** a + u * (smax ** a - smin ** a)) ** (1.0 / a)


def pixel_sources(rng, nsrc, npixel, cellsize, max_offset):
    """Source pixels (ix, iy) within +-max_offset rad of the centre; the
    direction cosines of pixel centres in RASCIL's convention
    (l = -(ix - n/2) cell, m = (iy - n/2) cell)."""
    half = min(int(max_offset / cellsize), npixel // 2 - 1)
    ix = npixel // 2 + rng.integers(-half, half + 1, nsrc)
    iy = npixel // 2 + rng.integers(-half, half + 1, nsrc)
    l = -(ix - npixel // 2) * cellsize
    m = (iy - npixel // 2) * cellsize
    return ix, iy, l, m


CONFIGS = {
    # Plain FP64 invert + predict round trip (CPU-runnable size)
    "small-array": dict(nants=64, layout=(("disk", 64, 1000.0),), lat=-26.7, dec=-45.0,
               freq=(100e6, 100e6, 1), ntimes=64, ha=(-2.0, 2.0), pol="stokesI",
               image_pol="stokesI", nsrc=20, flux=("uniform", 0.1, 1.0), offset=4.0,
               noise=0.0, npixel=512, cellsize=5e-4, epsilon=1e-12, dtype="c16"),
    # LOW-like: FP32 form vs plain FP64 form
    "low-like": dict(layout=(("disk", 224, 2000.0), ("lograd", 288, 2000.0, 35000.0)), lat=-26.7,
               dec=-30.0, freq=(100e6, 200e6, 16), ntimes=128, ha=(-3.0, 3.0), pol="linear",
               image_pol="stokesIQUV", nsrc=1000, flux=("powerlaw", 0.01, 1.0, 1.7),
               offset=2.0, noise=0.01, npixel=8192, cellsize=1e-5, epsilon=1e-5, dtype="c8"),
    # Differentiable predict geometry: 128 antennas drawn by the small array's law
    "gain-solve": dict(layout=(("disk", 128, 1000.0),), lat=-26.7, dec=-45.0,
               freq=(150e6, 158e6, 8), ntimes=64, ha=(-2.0, 2.0), pol="stokesI",
               image_pol="stokesI", nsrc=200, flux=("uniform", 0.01, 1.0), offset=4.0,
               noise=0.0, npixel=2048, cellsize=5e-4 / 4, epsilon=1e-5, dtype="c8"),
    # MID-like wide-field stress test
    "mid-like": dict(layout=(("disk", 64, 1000.0), ("lograd", 133, 1000.0, 80000.0)), lat=-30.7,
               dec=-60.0, freq=(0.95e9, 1.67e9, 64), ntimes=512, ha=(-4.0, 4.0), pol="linear",
               image_pol="stokesIQUV", nsrc=5000, flux=("uniform", 0.01, 1.0), offset=0.2,
               noise=0.0, npixel=16384, cellsize=5e-7, epsilon=1e-5, dtype="c8"),
}


def observation(name="small-array", seed=0, ntimes=None, nchan=None, npixel=None, nants=None):
    """Geometry of a named configuration: (uvw [ntimes, nbl, 3], freq,
    phasecentre, config dict).  Optional overrides shrink the case."""
    cfg = dict(CONFIGS[name])
    rng = numpy.random.default_rng(seed)
    east, north = [], []
    for spec in cfg["layout"]:
        if spec[0] == "disk":
            e, n = disk_positions(rng, spec[1], spec[2])
        else:
            e, n = log_radial_positions(rng, spec[1], spec[2], spec[3])
        east.append(e)
        north.append(n)
    east = numpy.concatenate(east)
    north = numpy.concatenate(north)
    if nants is not None:
        east, north = east[:nants], north[:nants]
    f0, f1, nf = cfg["freq"]
    if nchan is not None:
        nf = nchan
    freq = numpy.linspace(f0, f1, nf) if nf > 1 else numpy.array([f0])
    nt = ntimes or cfg["ntimes"]
    ha = numpy.linspace(cfg["ha"][0], cfg["ha"][1], nt) * numpy.pi / 12.0
    dec = numpy.radians(cfg["dec"])
    uvw = baseline_uvw(east, north, numpy.radians(cfg["lat"]), ha, dec)
    phasecentre = SkyDirection(0.0, dec)
    if npixel is not None:
        cfg["npixel"] = npixel
    return uvw, freq, phasecentre, cfg


def sources(cfg, seed=0):
    """Point sources snapped to pixel centres: (ix, iy, l, m, flux)."""
    rng = numpy.random.default_rng(seed + 1000)
    ix, iy, l, m = pixel_sources(rng, cfg["nsrc"], cfg["npixel"], cfg["cellsize"],
                                 numpy.radians(cfg["offset"]))
    kind = cfg["flux"][0]
    if kind == "uniform":
        flux = rng.uniform(cfg["flux"][1], cfg["flux"][2], cfg["nsrc"])
    else:
        flux = power_law_fluxes(rng, cfg["nsrc"], cfg["flux"][1], cfg["flux"][2], cfg["flux"][3])
    return ix, iy, l, m, flux


def model_image(cfg, src, phasecentre, freq):
    """MFS model image holding the sources' Stokes I at their pixels."""
    ix, iy, l, m, flux = src
    pol = PolarisationFrame(cfg["image_pol"])
    im = create_image(cfg["npixel"], cfg["cellsize"], phasecentre, frequency=[freq.mean()],
                      channel_bandwidth=[freq.max() - freq.min() + 1.0], polarisation_frame=pol)
    numpy.add.at(im["pixels"].data[0, 0], (numpy.asarray(iy, dtype=numpy.int64),
                                            numpy.asarray(ix, dtype=numpy.int64)),
                 numpy.asarray(flux, dtype=numpy.float64))
    return im


def component_fluxes(cfg, src, nchan):
    """[ncomp, nchan, npol] complex fluxes in the vis frame, divided by n so
    that the component DFT equals the image-plane operator (ducc0
    divides image pixels by n = sqrt(1 - l^2 - m^2))."""
    ix, iy, l, m, flux = src
    pol_img = PolarisationFrame(cfg["image_pol"])
    pol_vis = PolarisationFrame(cfg["pol"])
    stokes = numpy.zeros((len(flux), pol_img.npol), dtype=numpy.complex128)
    stokes[:, 0] = flux
    mat = conversion_matrix(pol_img, pol_vis)
    vf = stokes @ mat.T
    n = numpy.sqrt(1.0 - l * l - m * m)
    vf = vf / n[:, None]
    return numpy.repeat(vf[:, None, :], nchan, axis=1)


def lmn_rows(src):
    ix, iy, l, m, flux = src
    return numpy.stack([l, m, numpy.sqrt(1.0 - l * l - m * m) - 1.0], axis=-1)


def make_blockvisibility(uvw, freq, phasecentre, cfg, vis=None):
    pol = PolarisationFrame(cfg["pol"])
    nt, nbl, _ = uvw.shape
    if vis is None:
        dt = numpy.complex128 if cfg["dtype"] == "c16" else numpy.complex64
        vis = numpy.zeros((nt, nbl, len(freq), pol.npol), dtype=dt)
    return BlockVisibility(vis, uvw, freq, phasecentre, pol)


def snapshot_batch(nsnap=256, seed=0, min_vis=5000, max_vis=2_000_000,
                   sizes=(256, 512, 1024, 2048)):
    """Independent snapshots with uneven shapes (the batched configuration):
    each draws its own antenna count (32-512, positions uniform in a 1 km
    disk, latitude -26.7 deg, dec -45 deg), 1-8 channels inside 100-200 MHz,
    1-16 hour angles, an image side from ``sizes`` and a cell of
    1/(2.2 max|uv|); the visibility count is kept within [min_vis, max_vis]
    by trimming antennas.  Returns a list of dicts with uvw [ntimes, nbl, 3]
    (metres), freq, npix, cell."""
    rng = numpy.random.default_rng(seed + 77)
    out = []
    lat, dec = numpy.radians(-26.7), numpy.radians(-45.0)
    for s in range(nsnap):
        nant = int(rng.integers(32, 513))
        nchan = int(rng.integers(1, 9))
        ntimes = int(rng.integers(1, 17))
        while nant > 8 and nant * (nant - 1) // 2 * nchan * ntimes > max_vis:
            nant = int(nant * 0.9)
        while nant * (nant - 1) // 2 * nchan * ntimes < min_vis:
            ntimes += 1
        e, n = disk_positions(rng, nant, 1000.0)
        f_lo = rng.uniform(100e6, 190e6)
        f_hi = min(200e6, f_lo + rng.uniform(1e6, 50e6))
        freq = numpy.linspace(f_lo, f_hi, nchan) if nchan > 1 else numpy.array([f_lo])
        h0 = rng.uniform(-3.0, 2.0)
        ha = numpy.linspace(h0, h0 + rng.uniform(0.0, 1.0), ntimes) * numpy.pi / 12.0
        uvw = baseline_uvw(e, n, lat, ha, dec)
        uvmax = numpy.max(numpy.hypot(uvw[..., 0], uvw[..., 1])) * freq.max() / SPEED_OF_LIGHT
        npix = int(rng.choice(sizes))
        # 1/(2.2 max|uv|), but never past 0.6 rad from the centre (short
        # snapshots with large images would otherwise image beyond the horizon)
        cell = min(1.0 / (2.2 * uvmax), 0.6 / (npix / 2))
        out.append(dict(uvw=uvw, freq=freq, npix=npix, cell=cell,
                        nvis=uvw.shape[0] * uvw.shape[1] * nchan))
    return out
