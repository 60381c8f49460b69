"""Generate golden vectors by running the reference's own code.

Run in a checkout where the reference tree is available (its path is the
first argument, or RASCIL_REFERENCE_ROOT):

    python tests/golden/make_golden.py REFERENCE_ROOT

RASCIL itself cannot be imported here (astropy, xarray, ducc0 are absent),
so the functions on this path that are plain numpy are loaded directly:

* ``dft_cpu_looped`` -- extracted from
  ``rascil/processing_components/imaging/dft.py`` with ``ast`` and executed
  with numpy (the module's other imports are not needed by it);
* ``rascil/data_models/polarisation.py`` -- imported by file path (it needs
  only numpy);
* ``enu_to_xyz``, ``xyz_to_uvw``, ``simulate_point`` from
  ``rascil/processing_components/util/coordinate_support.py`` -- imported by
  file path with stand-in ``astropy`` modules (those three functions do not
  use astropy);
* ``normalise_sumwt`` -- extracted from
  ``rascil/processing_components/imaging/base.py`` with ``ast``;
* ``grid_blockvisibility_weight_to_griddata``,
  ``griddata_blockvisibility_reweight``, ``convolution_mapping_blockvisibility``
  and ``spatial_mapping`` -- extracted from
  ``rascil/processing_components/griddata/gridding.py`` with ``ast`` and run
  on stand-in BlockVisibility / GridData objects (the uv grid's WCS as the
  linear map create_griddata_from_image builds);
* ``phaserotate_visibility`` and ``calculate_blockvisibility_phasor`` --
  extracted from ``rascil/processing_components/visibility/base.py`` with
  ``ast`` and run on a stand-in BlockVisibility, with the reference's
  ``uvw_to_xyz`` / ``xyz_to_uvw`` and a direction-cosine stand-in for
  astropy's ``skycoord_to_lmn``.

Outputs go to ``tests/golden/*.npz`` next to this script.
"""
import ast
import copy
import importlib.util
import logging
import os
import sys
import types

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))


def load_function(path, name, namespace):
    tree = ast.parse(open(path).read(), filename=path)
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name == name:
            mod = ast.Module(body=[node], type_ignores=[])
            code = compile(mod, path, "exec")
            exec(code, namespace)
            return namespace[name]
    raise KeyError(name)


def load_module(path, name):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def stub_astropy():
    astropy = types.ModuleType("astropy")
    coords = types.ModuleType("astropy.coordinates")
    units = types.ModuleType("astropy.units")
    coords.SkyCoord = object
    coords.CartesianRepresentation = object
    astropy.coordinates = coords
    astropy.units = units
    sys.modules.setdefault("astropy", astropy)
    sys.modules.setdefault("astropy.coordinates", coords)
    sys.modules.setdefault("astropy.units", units)


def main(ref):
    rascil = os.path.join(ref, "rascil")
    rng = numpy.random.default_rng(20240601)

    # --- component DFT --------------------------------------------------------
    dft = load_function(os.path.join(rascil, "processing_components/imaging/dft.py"),
                        "dft_cpu_looped", {"numpy": numpy})
    ncomp, nt, nb, nch, npol = 7, 3, 11, 4, 4
    l = rng.uniform(-0.05, 0.05, ncomp)
    m = rng.uniform(-0.05, 0.05, ncomp)
    dirs = numpy.stack([l, m, numpy.sqrt(1 - l * l - m * m) - 1.0], axis=-1)
    uvw_lambda = rng.uniform(-2000, 2000, (nt, nb, nch, 3))
    vfluxes = (rng.uniform(0.1, 2.0, (ncomp, nch, npol))
               + 1j * rng.uniform(-0.1, 0.1, (ncomp, nch, npol)))
    vis = dft(dirs, uvw_lambda, vfluxes)
    numpy.savez_compressed(os.path.join(HERE, "dft_cpu_looped.npz"), direction_cosines=dirs,
                           uvw_lambda=uvw_lambda, vfluxes=vfluxes, vis=vis)

    # --- polarisation conversions ---------------------------------------------
    pol = load_module(os.path.join(rascil, "data_models/polarisation.py"), "ref_polarisation")
    pairs = [("linear", "stokesIQUV"), ("circular", "stokesIQUV"), ("stokesIQUV", "linear"),
             ("stokesIQUV", "circular"), ("linearnp", "stokesIQ"), ("circularnp", "stokesIV"),
             ("stokesIQ", "linearnp"), ("stokesIV", "circularnp"), ("linear", "stokesI"),
             ("circular", "stokesI"), ("linearnp", "stokesI"), ("circularnp", "stokesI"),
             ("stokesI", "stokesI")]
    out = {}
    for a, b in pairs:
        pa, pb = pol.PolarisationFrame(a), pol.PolarisationFrame(b)
        x = rng.normal(size=(5, 3, pa.npol)) + 1j * rng.normal(size=(5, 3, pa.npol))
        y = pol.convert_pol_frame(x, pa, pb, polaxis=2)
        out["in_%s_%s" % (a, b)] = x
        out["out_%s_%s" % (a, b)] = numpy.asarray(y)
    for name in pol.PolarisationFrame.polarisation_frames:
        out["names_%s" % name] = numpy.array(pol.PolarisationFrame(name).names)
    numpy.savez_compressed(os.path.join(HERE, "polarisation.npz"), **out)

    # --- geometry ----------------------------------------------------------------
    stub_astropy()
    cs = load_module(os.path.join(rascil, "processing_components/util/coordinate_support.py"),
                     "ref_coordinate_support")
    e = rng.uniform(-3000, 3000, 9)
    n = rng.uniform(-3000, 3000, 9)
    u = rng.uniform(-10, 10, 9)
    lat = numpy.radians(-26.7)
    x, y, z = cs.enu_to_xyz(e, n, u, lat)
    xyz = numpy.stack([x, y, z], axis=-1)
    has = numpy.linspace(-0.7, 0.9, 5)
    dec = numpy.radians(-45.0)
    uvw = numpy.stack([cs.xyz_to_uvw(xyz, h, dec) for h in has])
    dist = rng.uniform(-500, 500, (6, 2, 3))
    sp = cs.simulate_point(dist, 0.01, -0.02)
    numpy.savez_compressed(os.path.join(HERE, "geometry.npz"), e=e, n=n, u=u, lat=lat, xyz=xyz,
                           has=has, dec=dec, uvw=uvw, dist=dist, simulate_point=sp)

    # --- normalise_sumwt ---------------------------------------------------------
    ns = load_function(os.path.join(rascil, "processing_components/imaging/base.py"),
                       "normalise_sumwt", {"numpy": numpy, "Image": object, "log": logging})

    class _Img:
        def __init__(self, a):
            self._a = {"pixels": types.SimpleNamespace(data=a)}

        def __getitem__(self, k):
            return self._a[k]

    img = rng.normal(size=(2, 3, 8, 8))
    sumwt = numpy.array([[2.0, 0.0, 4.0], [-1.0, 8.0, 0.5]])
    res = ns(_Img(img.copy()), sumwt)["pixels"].data
    numpy.savez_compressed(os.path.join(HERE, "normalise_sumwt.npz"), image=img, sumwt=sumwt,
                           out=res)

    # --- imaging weights: weight gridding + reweighting --------------------------
    weighting_golden(rascil, rng)

    # --- phase rotation ----------------------------------------------------------
    rotation_golden(rascil, cs, rng)
    print("golden vectors written to", HERE)


class _LinearWcs:
    """Linear axes as astropy evaluates them for these grids:
    pixel = (world - crval) / cdelt + crpix - 1 (origin 0)."""

    def __init__(self, crpix, cdelt, crval):
        self.crpix = list(crpix)
        self.cdelt = list(cdelt)
        self.crval = list(crval)

    def sub(self, axes):
        i = [a - 1 for a in axes]
        return _LinearWcs([self.crpix[k] for k in i], [self.cdelt[k] for k in i],
                          [self.crval[k] for k in i])

    def wcs_world2pix(self, *args):
        world, origin = args[:-1], args[-1]
        return [(numpy.asarray(w) - self.crval[k]) / self.cdelt[k] + self.crpix[k] - 1 + origin * 0
                for k, w in enumerate(world)]


def weighting_golden(rascil, rng):
    """grid_blockvisibility_weight_to_griddata and
    griddata_blockvisibility_reweight (griddata/gridding.py) on stand-in
    BlockVisibility / GridData objects carrying exactly the attributes those
    functions read; the uv grid's WCS is the one create_griddata_from_image
    (griddata/operations.py:71-107) builds, as a linear _LinearWcs."""
    path = os.path.join(rascil, "processing_components/griddata/gridding.py")
    ns = {"numpy": numpy, "GridData": object}
    for fn in ("convolution_mapping_blockvisibility", "spatial_mapping",
               "grid_blockvisibility_weight_to_griddata", "griddata_blockvisibility_reweight"):
        load_function(path, fn, ns)
    grid_w = ns["grid_blockvisibility_weight_to_griddata"]
    reweight = ns["griddata_blockvisibility_reweight"]

    nt, nb, nch, npol, npix, nchan_img = 6, 9, 3, 2, 64, 3
    cell = 2.0e-3
    freq = numpy.array([1.0e8, 1.1e8, 1.25e8])
    uvmax = 0.45 / cell  # wavelengths: keep every sample inside the grid
    uvw = rng.uniform(-1.0, 1.0, (nt, nb, 3)) * numpy.array([1.0, 1.0, 0.2]) \
        * (uvmax * 299792458.0 / freq.max())
    weight = rng.uniform(0.5, 2.0, (nt, nb, nch, npol))
    imaging_weight = weight * rng.uniform(0.8, 1.2, weight.shape)
    flags = (rng.uniform(0, 1, weight.shape) < 0.1).astype(numpy.int64)
    # image WCS of a canonical image: RA---SIN cdelt -cell, DEC--SIN +cell (degrees),
    # frequency axis one channel per visibility channel
    cdelt_deg = numpy.degrees(cell)
    d2r = numpy.pi / 180.0
    cdu = 1.0 / (npix * -cdelt_deg * d2r)
    cdv = 1.0 / (npix * cdelt_deg * d2r)
    fwcs = _LinearWcs([1.0, 1.0, 1.0, 1.0], [cdu, cdv, 1.0, 1.0e7], [0.0, 0.0, 1.0, 1.0e8])
    fwcs.crpix = [npix // 2 + 1, npix // 2 + 1, 1.0, 1.0]
    fwcs.cdelt[3] = (freq[-1] - freq[0]) / (nchan_img - 1)
    fwcs.crval[3] = freq[0]
    k = freq / 299792458.0

    class _FlatArray(numpy.ndarray):
        """numpy 2 returns a read-only array from nan_to_num(a.flat); the
        reference was written against numpy 1, where it is a writable copy.
        .flat here gives that copy (same element order)."""

        @property
        def flat(self):
            return numpy.array(self).ravel()

    uvw_lambda = numpy.einsum("tbs,k->tbks", uvw, k).view(_FlatArray)

    class _BVisAcc:
        def __init__(self, v):
            self.v = v
            self.polarisation_frame = "pol"

        @property
        def flagged_imaging_weight(self):
            return self.v._d["imaging_weight"].data * (1 - self.v._d["flags"].data)

        @property
        def flagged_weight(self):
            return self.v._d["weight"].data * (1 - self.v._d["flags"].data)

    class _BVis:
        def __init__(self):
            self._d = {"imaging_weight": types.SimpleNamespace(data=imaging_weight.copy()),
                       "weight": types.SimpleNamespace(data=weight.copy()),
                       "flags": types.SimpleNamespace(data=flags.copy())}
            self.vis = types.SimpleNamespace(shape=weight.shape)
            self.frequency = types.SimpleNamespace(data=freq)
            self.uvw_lambda = types.SimpleNamespace(data=uvw_lambda)
            self.blockvisibility_acc = _BVisAcc(self)

        def __getitem__(self, key):
            return self._d[key]

    class _GridAcc:
        def __init__(self, gd):
            self.polarisation_frame = "pol"
            self.griddata_wcs = fwcs
            self.gd = gd

        @property
        def shape(self):
            return self.gd._d["pixels"].data.shape

    class _Grid:
        def __init__(self):
            self._d = {"pixels": types.SimpleNamespace(
                data=numpy.zeros((nchan_img, npol, npix, npix), dtype=complex))}
            self.griddata_acc = _GridAcc(self)

        def __getitem__(self, key):
            return self._d[key]

    # reweight reads vis.frequency (not .data) for the channel map
    out = {"uvw": uvw, "freq": freq, "weight": weight, "imaging_weight": imaging_weight,
           "flags": flags, "npix": npix, "cell": cell, "nchan_img": nchan_img,
           "wcs_crpix": numpy.array(fwcs.crpix), "wcs_cdelt": numpy.array(fwcs.cdelt),
           "wcs_crval": numpy.array(fwcs.crval)}
    for scheme, rob in (("uniform", 0.0), ("robust", 0.5), ("robust", -1.0), ("natural", 0.0)):
        vis = _BVis()
        gd, sumwt = grid_w(vis, _Grid())
        vis.frequency = freq
        res = reweight(vis, gd, weighting=scheme, robustness=rob)
        tag = "%s_%g" % (scheme, rob)
        out["grid_" + tag] = numpy.real(gd["pixels"].data)
        out["sumwt_" + tag] = sumwt
        out["imaging_weight_" + tag] = res["imaging_weight"].data
    numpy.savez_compressed(os.path.join(HERE, "weighting.npz"), **out)



def rotation_golden(rascil, cs, rng):
    """phaserotate_visibility with its phasor calculate_blockvisibility_phasor
    (visibility/base.py:296-357,1248-1264) on a stand-in BlockVisibility
    carrying exactly the attributes they read, with the reference's own
    uvw_to_xyz / xyz_to_uvw (util/coordinate_support.py).  skycoord_to_lmn
    (astropy) is replaced by the direction-cosine formula; the (l, m, n - 1)
    it gave are stored with the vectors, so a test can use the same ones."""
    path = os.path.join(rascil, "processing_components/visibility/base.py")
    lmn_used = {}

    def skycoord_to_lmn(pos, centre):
        ra, dec, ra0, dec0 = pos.ra.rad, pos.dec.rad, centre.ra.rad, centre.dec.rad
        l = numpy.cos(dec) * numpy.sin(ra - ra0)
        m = numpy.sin(dec) * numpy.cos(dec0) - numpy.cos(dec) * numpy.sin(dec0) * numpy.cos(ra - ra0)
        n = numpy.sin(dec) * numpy.sin(dec0) + numpy.cos(dec) * numpy.cos(dec0) * numpy.cos(ra - ra0)
        lmn_used["lmn"] = (l, m, n - 1.0)
        return l, m, n - 1.0

    def uvw_lambda(vis):
        vis.uvw_lambda.data = numpy.einsum("tbs,k->tbks", vis.uvw.data,
                                           vis.frequency.data / 299792458.0)
        return vis

    ns = {"numpy": numpy, "BlockVisibility": object, "SkyCoord": object,
          "skycoord_to_lmn": skycoord_to_lmn, "copy_visibility": copy.deepcopy,
          "uvw_to_xyz": cs.uvw_to_xyz, "xyz_to_uvw": cs.xyz_to_uvw,
          "calculate_blockvisibility_uvw_lambda": uvw_lambda}
    for fn in ("calculate_blockvisibility_phasor", "phaserotate_visibility"):
        load_function(path, fn, ns)
    rotate = ns["phaserotate_visibility"]

    class _Dir:
        def __init__(self, ra, dec):
            self.ra = types.SimpleNamespace(rad=ra)
            self.dec = types.SimpleNamespace(rad=dec)

    class _Arr:
        def __init__(self, a):
            self.data = a

        @property
        def shape(self):
            return self.data.shape

    class _BVis:
        def __init__(self, vis, uvw, freq, pc):
            self._v = {"vis": _Arr(vis), "uvw": _Arr(uvw)}
            self.frequency = _Arr(freq)
            self.uvw_lambda = _Arr(None)
            self.attrs = {"phasecentre": pc}
            uvw_lambda(self)

        def __getitem__(self, k):
            return self._v[k]

        @property
        def uvw(self):
            return self._v["uvw"]

        @property
        def vis(self):
            return self._v["vis"]

        @property
        def phasecentre(self):
            return self.attrs["phasecentre"]

    nt, nb, nch, npol = 3, 5, 4, 2
    freq = numpy.linspace(1.0e8, 1.3e8, nch)
    uvw = rng.uniform(-2000.0, 2000.0, (nt, nb, 3)) * numpy.array([1.0, 1.0, 0.15])
    vis = rng.normal(size=(nt, nb, nch, npol)) + 1j * rng.normal(size=(nt, nb, nch, npol))
    pc = (0.3, -0.6)
    new = (0.317, -0.585)
    out = dict(uvw=uvw, freq=freq, vis=vis, pc=numpy.array(pc), new=numpy.array(new))
    for tag, tangent, inverse in (("fwd", True, False), ("inv", True, True),
                                  ("fwd_nt", False, False), ("inv_nt", False, True)):
        b = _BVis(vis.copy(), uvw.copy(), freq, _Dir(*pc))
        r = rotate(b, _Dir(*new), tangent=tangent, inverse=inverse)
        out["vis_" + tag] = r["vis"].data
        out["uvw_" + tag] = r.uvw.data
    out["lmn"] = numpy.array(lmn_used["lmn"])
    numpy.savez_compressed(os.path.join(HERE, "rotation.npz"), **out)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RASCIL_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set RASCIL_REFERENCE_ROOT)")
    main(root)
