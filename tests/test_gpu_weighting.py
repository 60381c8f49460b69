"""GPU parity of the imaging weights (weight_visibility) against the CPU
restatement (oracle/weighting.py), which itself reproduces the reference's
own gridding.py functions bit for bit (tests/test_oracle.py).  Cells are
computed identically (the zero pattern and grid support must match
exactly); gridded sums and weights to 1e-12 relative (FP64 atomics add in
another order)."""
import os

import numpy
import pytest

from oracle import weighting as ow

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "weighting.npz")


def _make(uvw, freq, weight, imaging_weight, flags, npix, cell, nchan_img, pol):
    from rascil_gb300 import data_models as dm
    from rascil_gb300.polarisation import PolarisationFrame
    pc = dm.SkyDirection(0.0, numpy.radians(-45.0))
    f0, f1 = freq[0], freq[-1]
    img_freq = numpy.linspace(f0, f1, nchan_img) if nchan_img > 1 else numpy.array([f0])
    model = dm.create_image(npix, cell, pc, frequency=img_freq, nchan=nchan_img,
                            polarisation_frame=PolarisationFrame(pol))
    bvis = dm.BlockVisibility(numpy.zeros(weight.shape, numpy.complex64), uvw, freq, pc,
                              PolarisationFrame(pol), flags=flags.copy(), weight=weight.copy(),
                              imaging_weight=imaging_weight.copy())
    return bvis, model


def _oracle(bvis, model, scheme, rob):
    nt, nb, nch, npol = bvis.vis.shape
    sh = (nt * nb, nch, npol)
    wcs = model.image_acc.wcs
    v2i = numpy.round(wcs.sub([4]).wcs_world2pix(bvis.frequency.data, 0)[0]).astype(int)
    nci, _, ny, nx = model["pixels"].data.shape
    w, grid, sumwt = ow.weight_visibility(
        bvis.uvw.data, bvis.frequency.data, bvis["weight"].data.reshape(sh),
        bvis["imaging_weight"].data.reshape(sh), bvis["flags"].data.reshape(sh), v2i, nci, nx,
        ny, wcs.wcs.cdelt[0], wcs.wcs.cdelt[1], scheme, rob)
    return w.reshape(bvis.vis.shape)


CASES = [("uniform", 0.0), ("robust", 0.5), ("robust", -1.0), ("natural", 0.0)]


@pytest.mark.parametrize("scheme,rob", CASES)
def test_weights_match_reference_golden(scheme, rob):
    from rascil_gb300.imaging import weight_visibility
    d = numpy.load(GOLDEN)
    bvis, model = _make(d["uvw"], d["freq"], d["weight"], d["imaging_weight"], d["flags"],
                        int(d["npix"]), float(d["cell"]), int(d["nchan_img"]), "linearnp")
    got = weight_visibility(bvis, model, weighting=scheme, robustness=rob)["imaging_weight"].data
    ref = d["imaging_weight_%s_%g" % (scheme, rob)]
    numpy.testing.assert_array_equal(got == 0, ref == 0)
    numpy.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("scheme,rob", CASES)
def test_weights_larger_case_vs_oracle(scheme, rob):
    """The small array, 32 times, 4 channels onto 2 image channels,
    4 pols, 10 % flags, many samples per uv cell."""
    from rascil_gb300 import simulation as sim
    from rascil_gb300.imaging import weight_visibility
    uvw, _, pc, cfg = sim.observation("small-array", seed=3, ntimes=32)
    freq = numpy.linspace(1.0e8, 1.2e8, 4)
    rng = numpy.random.default_rng(11)
    shape = uvw.shape[:2] + (len(freq), 4)
    weight = rng.uniform(0.5, 2.0, shape)
    imw = weight * rng.uniform(0.8, 1.2, shape)
    flags = (rng.uniform(0, 1, shape) < 0.1).astype(numpy.int64)
    cell = 1.0 / (2.2 * numpy.max(numpy.abs(uvw[..., :2])) * freq.max() / 299792458.0)
    bvis, model = _make(uvw, freq, weight, imw, flags, 256, cell, 2, "linear")
    ref = _oracle(bvis, model, scheme, rob)
    got = weight_visibility(bvis, model, weighting=scheme, robustness=rob)["imaging_weight"].data
    numpy.testing.assert_array_equal(got == 0, ref == 0)
    numpy.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)


def test_out_of_grid_raises_like_the_reference_assert():
    from rascil_gb300 import _lib
    from rascil_gb300.imaging import weight_visibility
    d = numpy.load(GOLDEN)
    bvis, model = _make(d["uvw"], d["freq"], d["weight"], d["imaging_weight"], d["flags"],
                        int(d["npix"]), 5 * float(d["cell"]), int(d["nchan_img"]), "linearnp")
    with pytest.raises(AssertionError):
        weight_visibility(bvis, model, weighting="uniform")
    with pytest.raises(_lib.OutOfGridError):
        weight_visibility(bvis, model, weighting="robust")


def test_c_abi_rejects_unmapped_channels():
    """gb_weight_visibility checks the channel map before any launch."""
    import ctypes
    from rascil_gb300 import _lib
    lib = _lib.load()
    dev = torch.device("cuda")
    R, C, P, nci, n = 4, 2, 1, 1, 16
    uvw = torch.zeros((R, 3), dtype=torch.float64, device=dev)
    freq = torch.tensor([1e8, 1.1e8], dtype=torch.float64, device=dev)
    v2i = torch.tensor([0, 1], dtype=torch.int32, device=dev)  # channel 1 -> image channel 1 of 1
    w = torch.ones((R, C, P), dtype=torch.float64, device=dev)
    grid = torch.empty((nci, n, n, P), dtype=torch.float64, device=dev)
    cells = torch.empty((R, C), dtype=torch.int32, device=dev)
    out = torch.empty_like(w)
    sums = torch.empty(2, dtype=torch.float64, device=dev)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    rc = lib.gb_weight_visibility(p(uvw), p(freq), R, C, P, p(v2i), nci, n, n, -0.1, 0.1, p(w),
                                  p(w), None, _lib.GB_FLAGS_NONE, _lib.GB_WEIGHT_UNIFORM, 0.0,
                                  p(grid), p(cells), p(out), p(sums),
                                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.GB_ERR_INVALID_ARG
    assert b"image channel 1" in lib.gb_last_error_string()

