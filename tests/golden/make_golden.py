"""Generate golden vectors by running the reference's own code.

Run in a checkout where the reference tree is available (its path is the
first argument, default /root/reference):

    python tests/golden/make_golden.py /root/reference

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
  ``rascil/processing_components/imaging/base.py`` with ``ast``.

Outputs go to ``tests/golden/*.npz`` next to this script.
"""
import ast
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
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
