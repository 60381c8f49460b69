"""The oracle, pinned against the reference's own outputs and against
itself (CPU only)."""
import os

import numpy
import pytest

from oracle import dft
from oracle import wgridder as owg
from tests.cases import random_problem, rel_rms

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_component_dft_matches_reference_golden():
    """oracle.dft.dft_cpu_looped == the reference's dft_cpu_looped
    (rascil/processing_components/imaging/dft.py:261-281) on its golden run."""
    g = numpy.load(os.path.join(GOLDEN, "dft_cpu_looped.npz"))
    got = dft.dft_cpu_looped(g["direction_cosines"], g["uvw_lambda"], g["vfluxes"])
    numpy.testing.assert_allclose(got, g["vis"], rtol=0, atol=1e-12)


def test_image_operator_equals_component_dft_of_one_pixel():
    """dirty2ms on a one-pixel image, with ng.py's u/w flips and transpose,
    is the reference's component DFT of that pixel's direction with flux
    divided by n (ducc0 divides image pixels by n)."""
    rng = numpy.random.default_rng(3)
    npix, cell = 64, 1e-3
    uvw = rng.uniform(-1, 1, (50, 3)) * numpy.array([2000.0, 2000.0, 500.0])
    freq = numpy.array([1.0e8, 1.5e8])
    iy, ix = 17, 45  # RASCIL pixels[iy, ix]
    model = numpy.zeros((npix, npix))
    model[iy, ix] = 2.5
    fuvw = uvw * numpy.array([-1.0, 1.0, -1.0])
    got = dft.dirty2ms_dft(fuvw, freq, model.T, None, cell, cell, True)
    l = -(ix - npix // 2) * cell
    m = (iy - npix // 2) * cell
    n = numpy.sqrt(1 - l * l - m * m)
    uvw_lambda = uvw[:, None, :] * (freq / dft.SPEED_OF_LIGHT)[None, :, None]
    ref = dft.dft_cpu_looped(numpy.array([[l, m, n - 1.0]]), uvw_lambda[None],
                             numpy.full((1, 2, 1), 2.5 / n, dtype=complex))[0, ..., 0]
    numpy.testing.assert_allclose(got, ref, rtol=0, atol=1e-12)


def test_ms2dirty_and_dirty2ms_are_adjoint():
    c = random_problem(seed=11, nrow=60, npix=32)
    ms, img = c["ms"][..., 0], c["img"][0]
    a = dft.ms2dirty_dft(c["uvw"], c["freq"], ms, None, 32, 32, c["pixsize"], c["pixsize"], True)
    b = dft.dirty2ms_dft(c["uvw"], c["freq"], img, None, c["pixsize"], c["pixsize"], True)
    lhs = numpy.sum(a * img)
    rhs = numpy.real(numpy.vdot(b, ms))
    assert abs(lhs - rhs) < 1e-9 * abs(lhs)


@pytest.mark.parametrize("do_w", [False, True])
@pytest.mark.parametrize("eps,tol", [(1e-5, 1e-5), (1e-12, 1e-10)])
def test_numpy_gridder_matches_dft(do_w, eps, tol):
    c = random_problem(seed=12, nrow=150)
    ms, wgt, img = c["ms"][..., 0], c["wgt"][..., 0], c["img"][0]
    ref = dft.ms2dirty_dft(c["uvw"], c["freq"], ms, wgt, 64, 64, c["pixsize"], c["pixsize"], do_w)
    got = owg.ms2dirty(c["uvw"], c["freq"], ms, wgt, 64, 64, c["pixsize"], c["pixsize"], eps, do_w)
    assert rel_rms(got, ref) < tol
    vref = dft.dirty2ms_dft(c["uvw"], c["freq"], img, None, c["pixsize"], c["pixsize"], do_w)
    vgot = owg.dirty2ms(c["uvw"], c["freq"], img, None, c["pixsize"], c["pixsize"], eps, do_w)
    assert rel_rms(vgot, vref) < tol


@pytest.mark.parametrize("do_w", [False, True])
def test_c_gridder_matches_numpy_gridder(do_w):
    from oracle import cgridder
    c = random_problem(seed=13, nrow=300)
    ms, wgt, img = c["ms"][..., 0], c["wgt"][..., 0], c["img"][0]
    a = owg.ms2dirty(c["uvw"], c["freq"], ms, wgt, 64, 64, c["pixsize"], c["pixsize"], 1e-12, do_w)
    b = cgridder.ms2dirty(c["uvw"], c["freq"], ms, wgt, 64, 64, c["pixsize"], c["pixsize"], 1e-12,
                          do_w, nthreads=4)
    assert rel_rms(b, a) < 1e-13
    va = owg.dirty2ms(c["uvw"], c["freq"], img, None, c["pixsize"], c["pixsize"], 1e-12, do_w)
    vb = cgridder.dirty2ms(c["uvw"], c["freq"], img, None, c["pixsize"], c["pixsize"], 1e-12,
                           do_w, nthreads=4)
    assert rel_rms(vb, va) < 1e-13


def test_c_gridder_plane_subset_sums_to_whole():
    """The bench's bounded CPU sample grids a subset of w-planes; the parts
    over a partition of the planes add up to the full result."""
    from oracle import cgridder
    c = random_problem(seed=14, nrow=200)
    ms = c["ms"][..., 0]
    pr = cgridder.Prepared.from_uvw(c["uvw"], c["freq"], 64, 64, c["pixsize"], c["pixsize"],
                                    1e-5, True)
    full = cgridder.grid_items(pr, ms, 2)
    k = pr.plan.nplanes
    parts = cgridder.grid_items(pr, ms, 2, range(0, k, 2)) + cgridder.grid_items(pr, ms, 2,
                                                                                  range(1, k, 2))
    assert rel_rms(parts, full) < 1e-13


def test_weighting_oracle_matches_reference_golden():
    """oracle/weighting.py reproduces the reference's own
    grid_blockvisibility_weight_to_griddata + griddata_blockvisibility_reweight
    (tests/golden/weighting.npz, made by tests/golden/make_golden.py)."""
    import os
    import numpy
    from oracle import weighting as ow
    d = numpy.load(os.path.join(os.path.dirname(__file__), "golden", "weighting.npz"))
    npix, cell, nchan_img = int(d["npix"]), float(d["cell"]), int(d["nchan_img"])
    nt, nb, nch, npol = d["weight"].shape
    crpix, cdelt, crval = d["wcs_crpix"], d["wcs_cdelt"], d["wcs_crval"]
    freq = d["freq"]
    vis_to_im = numpy.round((freq - crval[3]) / cdelt[3] + crpix[3] - 1).astype(int)
    cdelt_deg = numpy.degrees(cell)
    sh = (nt * nb, nch, npol)
    for scheme, rob in (("uniform", 0.0), ("robust", 0.5), ("robust", -1.0), ("natural", 0.0)):
        tag = "%s_%g" % (scheme, rob)
        w, grid, sumwt = ow.weight_visibility(
            d["uvw"], freq, d["weight"].reshape(sh), d["imaging_weight"].reshape(sh),
            d["flags"].reshape(sh), vis_to_im, nchan_img, npix, npix, -cdelt_deg, cdelt_deg,
            scheme, rob)
        numpy.testing.assert_array_equal(grid, d["grid_" + tag])
        numpy.testing.assert_array_equal(sumwt, d["sumwt_" + tag])
        numpy.testing.assert_array_equal(w.reshape(d["weight"].shape), d["imaging_weight_" + tag])


def test_rotation_oracle_matches_reference_golden():
    """phaserotate_visibility / calculate_blockvisibility_phasor run from the
    reference's own source (tests/golden/make_golden.py) on the same (l, m,
    n - 1): forward, inverse, and the tangent=False variants (same vis)."""
    from oracle import rotation as orot
    g = numpy.load(os.path.join(GOLDEN, "rotation.npz"))
    for tag, inverse in (("fwd", False), ("inv", True), ("fwd_nt", False), ("inv_nt", True)):
        got = orot.phaserotate(g["vis"], g["uvw"], g["freq"], g["lmn"], inverse=inverse)
        numpy.testing.assert_allclose(got, g["vis_" + tag], rtol=0, atol=1e-12)
    u = orot.rotate_uvw(g["uvw"], *g["pc"], *g["new"])
    numpy.testing.assert_allclose(u, g["uvw_fwd_nt"], rtol=0, atol=1e-9)
    geo = numpy.load(os.path.join(GOLDEN, "geometry.npz"))
    numpy.testing.assert_allclose(orot.simulate_point(geo["dist"], 0.01, -0.02),
                                  geo["simulate_point"], rtol=0, atol=1e-12)



def test_c_gridder_threads_give_the_serial_result():
    """The oracle's C gridder grids row bands in two parity passes; with
    every band the same height and an even number of them, supports that
    wrap from the last band into band 0 never race (1280-row grids at
    sigma 1.25 once did), so any thread count gives the serial image."""
    from oracle import cgridder
    from tests.cases import random_problem
    c = random_problem(seed=3, nrow=4000, nchan=2, npix=1024, pixsize=4e-4, wscale=400.0,
                       uvscale=1200.0)
    args = (c["uvw"], c["freq"], c["ms"][..., 0], None, 1024, 1024, 4e-4, 4e-4, 1e-5, True)
    one = cgridder.ms2dirty(*args, nthreads=1, sigma=1.25)
    many = cgridder.ms2dirty(*args, nthreads=8, sigma=1.25)
    numpy.testing.assert_array_equal(one, many)
