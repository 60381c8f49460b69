"""Host-side logic of the product (CPU only): pol matrices, geometry,
normalisation, the data-model shim, the planner through the C-ABI (no
GPU), the symbol table and argument errors."""
import ctypes
import os
import re

import numpy
import pytest

from tests.cases import rel_rms

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def test_polarisation_matches_reference_golden():
    from rascil_gb300.polarisation import PolarisationFrame, convert_pol_frame
    g = numpy.load(os.path.join(GOLDEN, "polarisation.npz"))
    pairs = sorted({k[3:] for k in g.files if k.startswith("in_")})
    assert len(pairs) == 13
    for pair in pairs:
        a, b = pair.split("_")
        got = convert_pol_frame(g["in_" + pair], PolarisationFrame(a), PolarisationFrame(b),
                                polaxis=2)
        numpy.testing.assert_allclose(got, g["out_" + pair], rtol=0, atol=1e-15, err_msg=pair)
    for k in g.files:
        if k.startswith("names_"):
            assert PolarisationFrame(k[6:]).names == list(g[k])


def test_unknown_conversion_raises():
    from rascil_gb300.polarisation import conversion_matrix
    with pytest.raises(ValueError):
        conversion_matrix("linear", "circular")


def test_geometry_matches_reference_golden():
    from rascil_gb300 import simulation as sim
    g = numpy.load(os.path.join(GOLDEN, "geometry.npz"))
    x, y, z = sim.enu_to_xyz(g["e"], g["n"], g["u"], float(g["lat"]))
    numpy.testing.assert_allclose(numpy.stack([x, y, z], -1), g["xyz"], rtol=0, atol=1e-9)
    uvw = numpy.stack([sim.xyz_to_uvw(g["xyz"], h, float(g["dec"])) for h in g["has"]])
    numpy.testing.assert_allclose(uvw, g["uvw"], rtol=0, atol=1e-9)


def test_baseline_counts_of_named_configurations():
    from rascil_gb300 import simulation as sim
    for name, nbl in (("small-array", 2016), ("low-like", 130816), ("gain-solve", 8128), ("mid-like", 19306)):
        uvw, f, pc, cfg = sim.observation(name, ntimes=1)
        assert uvw.shape == (1, nbl, 3)


def test_normalise_sumwt_matches_reference_golden():
    from rascil_gb300.data_models import Image, WCS
    from rascil_gb300.imaging.base import normalise_sumwt
    from rascil_gb300.polarisation import PolarisationFrame
    g = numpy.load(os.path.join(GOLDEN, "normalise_sumwt.npz"))
    im = Image(g["image"].copy(), WCS(["RA---SIN", "DEC--SIN", "STOKES", "FREQ"], [5, 5, 1, 1],
                                      [-1, 1, 1, 1], [0, 0, 1, 1]),
               PolarisationFrame("stokesI"), None)
    out = normalise_sumwt(im, g["sumwt"])["pixels"].data
    numpy.testing.assert_array_equal(out, g["out"])


def test_blockvisibility_shim_accessors():
    from rascil_gb300 import simulation as sim
    from rascil_gb300.data_models import copy_visibility
    uvw, f, pc, cfg = sim.observation("small-array", ntimes=2)
    b = sim.make_blockvisibility(uvw, f, pc, cfg)
    b["vis"].data[...] = 1 + 2j
    b["flags"].data[0, 0, 0, 0] = 1
    b["imaging_weight"].data[...] = 3.0
    assert b.blockvisibility_acc.flagged_vis[0, 0, 0, 0] == 0
    assert b.blockvisibility_acc.flagged_vis[1, 0, 0, 0] == 1 + 2j
    assert b.blockvisibility_acc.flagged_imaging_weight[0, 0, 0, 0] == 0
    z = copy_visibility(b, zero=True)
    assert numpy.all(z["vis"].data == 0) and numpy.all(b["vis"].data == 1 + 2j)
    assert b.vis.shape == (2, 2016, 1, 1)


def test_image_wcs_and_phase_centre():
    from rascil_gb300 import simulation as sim
    from rascil_gb300.imaging.base import image_is_canonical, image_phasecentre, separation
    uvw, f, pc, cfg = sim.observation("small-array", ntimes=1)
    im = sim.model_image(cfg, sim.sources(cfg), pc, f)
    assert image_is_canonical(im)
    assert separation(image_phasecentre(im), pc) < 1e-15
    ch = im.image_acc.wcs.sub([4]).wcs_world2pix(f, 0)[0]
    numpy.testing.assert_allclose(ch, 0.0)


def test_lmn_known_answers():
    """skycoord_to_lmn's known answers (reference
    tests/processing_components/test_coordinate_support.py:139-155), as
    (l, m, n - 1)."""
    from rascil_gb300.data_models import SkyDirection
    from rascil_gb300.imaging.base import lmn_of
    d = numpy.radians
    centre, north, south = SkyDirection(0, 0), SkyDirection(0, d(90)), SkyDirection(0, d(-90))
    east, west = SkyDirection(d(90), 0), SkyDirection(d(-90), 0)
    cases = [(centre, centre, (0, 0, 0)), (north, centre, (0, 1, -1)),
             (south, centre, (0, -1, -1)), (south, north, (0, 0, -2)),
             (east, centre, (1, 0, -1)), (west, centre, (-1, 0, -1)),
             (centre, west, (1, 0, -1)), (north, west, (0, 1, -1)),
             (south, west, (0, -1, -1)), (north, east, (0, 1, -1)),
             (south, east, (0, -1, -1))]
    for pos, ctr, want in cases:
        l, m, n = lmn_of(pos, ctr)
        numpy.testing.assert_allclose((l, m, n - 1.0), want, atol=1e-14)


def test_uvw_rotation_matches_reference_golden():
    """tangent=False uvw rotation (visibility/base.py:331-355, the
    reference's uvw_to_xyz / xyz_to_uvw)."""
    from rascil_gb300.data_models import SkyDirection
    from rascil_gb300.imaging.base import _rotate_uvw
    g = numpy.load(os.path.join(GOLDEN, "rotation.npz"))
    got = _rotate_uvw(g["uvw"].reshape(-1, 3), SkyDirection(*g["pc"]), SkyDirection(*g["new"]))
    numpy.testing.assert_allclose(got.reshape(g["uvw"].shape), g["uvw_fwd_nt"], rtol=0,
                                  atol=1e-9)


def test_phase_rotation_property_of_rotated_uvw():
    """The reference's test_phase_rotate (test_coordinate_support.py:157-193):
    a point source seen from phase centre A, times the phasor of A about B
    on B's uvw, equals the same source seen from B."""
    from oracle.rotation import simulate_point
    from rascil_gb300.data_models import SkyDirection
    from rascil_gb300.imaging.base import _rotate_uvw, lmn_of
    uvw = numpy.array([(1.0, 0, 0), (0, 1.0, 0), (0, 0, 1.0)])
    d = numpy.radians
    pos = [SkyDirection(d(17), d(35)), SkyDirection(d(17), d(30)), SkyDirection(d(12), d(30)),
           SkyDirection(d(11), d(35)), SkyDirection(d(51), d(35)), SkyDirection(d(15), d(70))]
    for pc in pos:
        for new in pos:
            uvw_r = _rotate_uvw(uvw, pc, new)
            lp, mp, _ = lmn_of(pc, new)
            ph = simulate_point(uvw_r, lp, mp)
            for src in pos:
                l, m, _ = lmn_of(src, pc)
                lr, mr, _ = lmn_of(src, new)
                numpy.testing.assert_allclose(simulate_point(uvw, l, m) * ph,
                                              simulate_point(uvw_r, lr, mr), atol=1e-10)


def test_fused_phase_shift_is_the_plan_frame_direction():
    """invert_ng / predict_ng fuse shift_vis_to_image into the plan: the
    shift is (-l, m, -(sqrt(1 - l^2 - m^2) - 1)) because ng.py hands the
    gridder uvw with u and w negated; none when the centres agree."""
    from rascil_gb300 import simulation as sim
    from rascil_gb300.data_models import SkyDirection
    from rascil_gb300.imaging.base import fused_phase_shift, lmn_of
    uvw, f, pc, cfg = sim.observation("small-array", ntimes=1)
    b = sim.make_blockvisibility(uvw, f, pc, cfg)
    im = sim.model_image(cfg, ([], [], [], [], []), pc, f)
    assert fused_phase_shift(b, im) == (False, (0.0, 0.0, 0.0))
    off = SkyDirection(pc.ra.rad + 0.01, pc.dec.rad - 0.005)
    im = sim.model_image(cfg, ([], [], [], [], []), off, f)
    rot, s = fused_phase_shift(b, im)
    l, m, _ = lmn_of(off, pc)
    assert rot
    numpy.testing.assert_allclose(s, (-l, m, -(numpy.sqrt(1 - l * l - m * m) - 1.0)),
                                  rtol=1e-14, atol=0)


def _header_functions():
    text = open(os.path.join(ROOT, "include", "rascil_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from rascil_gb300 import _lib
    lib = _lib.load()
    names = _header_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name


@pytest.mark.parametrize("case", [
    dict(npix_x=63), dict(npol=3), dict(epsilon=1e-8, precision="fp32"),
    dict(pixsize_x=0.01), dict(sigma=1.9), dict(epsilon=1e-16, precision="fp64"),
    dict(nrows=1 << 31, nchan=2)])
def test_planner_rejects_invalid_arguments(case):
    """Including more than 2^32 - 1 (row, channel) items in one plan: the
    item index is 32-bit, so such a call must be split."""
    from rascil_gb300.wgridder import plan_geometry
    kw = dict(npix_x=256, npix_y=256, pixsize_x=1e-3, pixsize_y=1e-3, epsilon=1e-5,
              do_wstacking=True, w_lo=-100.0, w_hi=200.0, precision="fp32", npol=1)
    kw.update(case)
    with pytest.raises(ValueError):
        plan_geometry(**kw)


@pytest.mark.parametrize("precision,eps", [("fp64", 1e-12), ("fp32", 1e-5), ("fp64", 1e-7)])
@pytest.mark.parametrize("do_w", [False, True])
@pytest.mark.parametrize("npix,cell", [(512, 5e-4), (8192, 1e-5), (250, 2e-3)])
def test_planner_geometry_matches_oracle(precision, eps, do_w, npix, cell):
    """The C planner (host only) and the oracle's restatement agree exactly."""
    from oracle import wgridder as owg
    from rascil_gb300.wgridder import plan_geometry
    w_lo, w_hi = -1234.5, 4321.25
    info = plan_geometry(npix, npix, cell, cell, eps, do_w, w_lo, w_hi, precision=precision,
                         sigma=2.0)
    op = owg.Plan(npix, npix, cell, cell, eps, do_w, w_lo, w_hi, fp32=precision == "fp32")
    assert info["support"] == op.W and info["beta"] == op.beta
    assert info["ngrid_x"] == op.ngx and info["ngrid_y"] == op.ngy
    assert info["nplanes"] == op.nplanes
    if do_w:
        assert info["dw"] == op.dw and info["tc"] == op.tc


def test_es_table_kernel_choice_is_monotone():
    from oracle.wgridder import es_table
    rows = es_table()
    for s in (1.25, 1.5, 1.75, 2.0):
        errs = [e for (ss, w, b, e) in rows if ss == s]
        assert len(errs) == 13
        assert errs[-1] < errs[0] * 1e-6


def test_weighting_rejects_channels_outside_the_image():
    """A visibility channel that maps outside the image's channels raises
    before any device work, as the reference's numpy indexing does."""
    from rascil_gb300 import data_models as dm
    from rascil_gb300 import simulation as sim
    from rascil_gb300.imaging import weight_visibility
    uvw, f, pc, cfg = sim.observation("small-array", ntimes=1)
    f = numpy.array([1.0e8, 1.5e8])
    b = sim.make_blockvisibility(uvw, f, pc, cfg)
    model = dm.create_image(64, 1e-3, pc, frequency=[1.0e8], channel_bandwidth=[1e6])
    with pytest.raises(IndexError):
        weight_visibility(b, model)


def test_copy_visibility_keeps_aliases_and_takes_given_vis():
    """copy_visibility deep-copies every array once: arrays the input shares
    (weight and imaging_weight as one array, as natural weighting leaves
    them) stay shared in the copy and independent of the input; a given vis
    array becomes the copy's visibilities without a copy."""
    from rascil_gb300 import simulation as sim
    from rascil_gb300.data_models import BlockVisibility, copy_visibility
    uvw, f, pc, cfg = sim.observation("small-array", ntimes=2)
    shape = uvw.shape[:2] + (len(f), 1)
    w = numpy.full(shape, 2.0)
    b = BlockVisibility(numpy.ones(shape, numpy.complex128), uvw, f, pc,
                        sim.PolarisationFrame("stokesI"), weight=w, imaging_weight=w)
    c = copy_visibility(b)
    assert c["weight"].data is c["imaging_weight"].data
    assert c["weight"].data is not w
    c["imaging_weight"].data[...] = 5.0
    assert numpy.all(w == 2.0) and numpy.all(c["weight"].data == 5.0)
    given = numpy.zeros(shape, numpy.complex128)
    d = copy_visibility(b, vis=given)
    assert d["vis"].data is given and d.uvw.data is not b.uvw.data
    z = copy_visibility(b, zero=True)
    assert numpy.all(z["vis"].data == 0) and numpy.all(b["vis"].data == 1)
    assert c.phasecentre is not None and c.attrs is not b.attrs
    # predict_ng's form: every array but vis copied, vis left for the caller
    s = copy_visibility(b, skip_vis=True)
    assert s["vis"].data is None and s["weight"].data is s["imaging_weight"].data
    assert s["weight"].data is not w and numpy.all(s["flags"].data == b["flags"].data)
    s["vis"].data = given
    assert s.vis.shape == b.vis.shape


def test_empty_visibilities_need_no_device():
    """No samples: invert_ng gives a zero image and zero weight sums,
    predict_ng a zeroed copy, weight_visibility leaves the (empty) weights --
    what the reference's ducc0 calls and numpy loops give -- before any
    device work."""
    from rascil_gb300 import simulation as sim
    from rascil_gb300.imaging import invert_ng, predict_ng, weight_visibility
    uvw, f, pc, cfg = sim.observation("small-array", ntimes=1, npixel=64)
    b = sim.make_blockvisibility(uvw[:0], f, pc, cfg)
    model = sim.model_image(cfg, ([], [], [], [], []), pc, f)
    model["pixels"].data[...] = 1.0
    im, sw = invert_ng(b, model)
    assert numpy.all(im["pixels"].data == 0) and numpy.all(sw == 0)
    assert im["pixels"].data.shape == model["pixels"].data.shape
    assert numpy.all(model["pixels"].data == 1.0)
    p = predict_ng(b, model)
    assert p is not b and p["vis"].data.shape == b["vis"].data.shape
    assert weight_visibility(b, model) is b


@pytest.mark.parametrize("sigma", [1.25, 1.5, 1.75])
def test_planner_geometry_matches_oracle_other_sigmas(sigma):
    from oracle import wgridder as owg
    from rascil_gb300.wgridder import plan_geometry
    prec = "fp64" if sigma < 1.5 else "fp32"  # the FP32 form keeps sigma >= 1.5
    info = plan_geometry(1024, 1024, 1e-4, 1e-4, 1e-5, True, -800.0, 2500.0, precision=prec,
                         sigma=sigma)
    op = owg.Plan(1024, 1024, 1e-4, 1e-4, 1e-5, True, -800.0, 2500.0, sigma=sigma,
                  fp32=prec == "fp32")
    assert (info["support"], info["beta"], info["ngrid_x"], info["nplanes"], info["dw"]) == (
        op.W, op.beta, op.ngx, op.nplanes, op.dw)


def test_planner_chooses_oversampling_by_cost():
    """With sigma 0 the planner weighs gridding work (W^3 per item) against
    per-plane transform work: a wide field with few visibilities and many
    w-planes whose image side is not a power of two (cuFFT transforms at
    every oversampling) takes the smallest oversampling its form allows
    (1.5 for FP32, whose grid rounding sigma 1.25's edge correction would
    amplify beyond epsilon); with a power-of-two side the FP32 form keeps
    sigma 2, whose grids take the library's pruned column transforms
    (measured faster than sigma 1.5's smaller cuFFT grids); a dense narrow
    field (the LOW-like workload) keeps sigma 2; an explicit sigma is kept."""
    from rascil_gb300.wgridder import plan_geometry
    wide = plan_geometry(1800, 1800, 6.6e-4, 6.6e-4, 1e-5, True, -700.0, 700.0, nrows=100000,
                         nchan=2, precision="fp32")
    assert wide["sigma"] == 1.5 and wide["fft_mode"] == 1  # 1.25 is below the FP32 form's
    wide2 = plan_geometry(2048, 2048, 5.8e-4, 5.8e-4, 1e-5, True, -700.0, 700.0, nrows=100000,
                          nchan=2, precision="fp32")
    assert wide2["sigma"] == 2.0 and wide2["fft_mode"] == 2
    wide64 = plan_geometry(2048, 2048, 5.8e-4, 5.8e-4, 1e-7, True, -700.0, 700.0, nrows=100000,
                           nchan=2, precision="fp64")
    assert wide64["sigma"] == 1.25
    dense = plan_geometry(8192, 8192, 1e-5, 1e-5, 1e-5, True, -40000.0, 41000.0,
                          nrows=16744448, nchan=16, npol=4, precision="fp32")
    assert dense["sigma"] == 2.0 and dense["fft_mode"] == 2
    fixed = plan_geometry(2048, 2048, 5.8e-4, 5.8e-4, 1e-5, True, -700.0, 700.0, nrows=100000,
                          nchan=2, precision="fp32", sigma=2.0)
    assert fixed["sigma"] == 2.0
