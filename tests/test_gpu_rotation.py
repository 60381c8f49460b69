"""GPU parity of the tangent-plane phase rotation.

* ``phaserotate_visibility`` / ``shift_vis_to_image`` (``gb_phase_rotate``)
  against the reference's own output (``tests/golden/rotation.npz``) and
  the oracle (``oracle/rotation.py``);
* the rotation fused into the gridder plans: ``invert_ng`` with an image
  centred away from the visibilities' phase centre equals ``invert_ng`` of
  the oracle-rotated visibilities with a centred image (what the
  reference's ``shift_vis_to_image`` at ng.py:169-170 does), its PSF
  ignores the shift (the reference sets unit visibilities after rotating),
  and ``predict_ng`` equals the centred prediction times the inverse
  phasor (ng.py:129-130).

Tolerances: FP64 kernels 1e-12 (absolute on unit-scale data, or relative
RMS); FP32 data within complex64 rounding (2e-6) for the rotation alone and
1e-5 relative RMS (the FP32 form's accuracy bar) through the gridder.
"""
import os

import numpy
import pytest

from oracle import rotation as orot
from oracle.dft import lmn_of_direction
from tests.cases import rel_rms

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "rotation.npz")


def _golden_bvis(dtype=numpy.complex128):
    from rascil_gb300 import data_models as dm
    from rascil_gb300.polarisation import PolarisationFrame
    g = numpy.load(GOLDEN)
    bvis = dm.BlockVisibility(g["vis"].astype(dtype), g["uvw"].copy(), g["freq"],
                              dm.SkyDirection(*g["pc"]), PolarisationFrame("linearnp"))
    return g, bvis


@pytest.mark.parametrize("tag,tangent,inverse", [("fwd", True, False), ("inv", True, True),
                                                 ("fwd_nt", False, False),
                                                 ("inv_nt", False, True)])
def test_phaserotate_matches_reference_golden(tag, tangent, inverse):
    from rascil_gb300.data_models import SkyDirection
    from rascil_gb300.imaging.base import phaserotate_visibility
    g, bvis = _golden_bvis()
    new = SkyDirection(*g["new"])
    out = phaserotate_visibility(bvis, new, tangent=tangent, inverse=inverse)
    assert out is not bvis
    numpy.testing.assert_allclose(out["vis"].data, g["vis_" + tag], rtol=0, atol=1e-12)
    numpy.testing.assert_allclose(out.uvw.data, g["uvw_" + tag], rtol=0, atol=1e-9)
    numpy.testing.assert_array_equal(bvis["vis"].data, g["vis"])  # input untouched
    if not tangent:
        assert out.phasecentre is new
    # complex64 data: the same rotation within complex64 rounding
    g, b64 = _golden_bvis(numpy.complex64)
    out = phaserotate_visibility(b64, new, tangent=tangent, inverse=inverse)
    assert out["vis"].data.dtype == numpy.complex64
    ref = g["vis_" + tag]
    assert numpy.max(numpy.abs(out["vis"].data - ref)) < 2e-6 * numpy.max(numpy.abs(ref))


@pytest.mark.parametrize("dtype,rel,per_turn", [(numpy.complex128, 1e-14, 1e-14),
                                                (numpy.complex64, 1e-6, 0.0)])
def test_phaserotate_kernel_matches_oracle_at_size(dtype, rel, per_turn):
    """200,000 rows x 8 channels x 4 pols, baselines up to 60 km (phases of
    up to ~2,000 turns), both directions.  FP64 fixes a phase summed from
    terms of size T turns only to ~T 2^-52 turns, so the complex128 bound
    grows with T = |u l| + |v m| + |w (n - 1)| (2 pi T 1e-14 |vis|, about 40
    ulps of the phase); complex64: 1e-6 |vis|."""
    from rascil_gb300 import data_models as dm
    from rascil_gb300.imaging.base import phaserotate_visibility
    from rascil_gb300.polarisation import PolarisationFrame
    rng = numpy.random.default_rng(5)
    R, C, P = 200_000, 8, 4
    uvw = rng.uniform(-6e4, 6e4, (R, 1, 3)) * numpy.array([1.0, 1.0, 0.1])
    freq = numpy.linspace(1.0e8, 2.0e8, C)
    vis = (rng.normal(size=(R, 1, C, P)) + 1j * rng.normal(size=(R, 1, C, P))).astype(dtype)
    pc = dm.SkyDirection(1.1, -0.4)
    new = dm.SkyDirection(1.13, -0.43)
    bvis = dm.BlockVisibility(vis, uvw, freq, pc, PolarisationFrame("linear"))
    l, m, n = lmn_of_direction(new.ra.rad, new.dec.rad, pc.ra.rad, pc.dec.rad)
    for inverse in (False, True):
        got = phaserotate_visibility(bvis, new, inverse=inverse)["vis"].data
        ref = orot.phaserotate(vis.astype(numpy.complex128), uvw, freq, (l, m, n - 1.0),
                               inverse=inverse)
        # magnitude of the phase's terms |u l| + |v m| + |w (n - 1)| (turns)
        turns = (numpy.abs(uvw[..., None, :]) * (freq / 299792458.0)[:, None]
                 @ numpy.abs(orot.direction(l, m)))[..., None]
        bound = numpy.abs(vis) * (rel + 2 * numpy.pi * turns * per_turn)
        assert numpy.all(numpy.abs(got - ref) <= bound)


def test_shift_vis_to_image_to_offset_image_centre():
    """shift_vis_to_image multiplies by conj(exp(-2 pi i uvw_lambda.(l, m, n-1)))
    of the image centre, relabels the phase centre, and is a no-op once the
    centres agree (imaging/base.py:67-106)."""
    from rascil_gb300 import simulation as sim
    from rascil_gb300.data_models import SkyDirection
    from rascil_gb300.imaging.base import lmn_of, shift_vis_to_image
    uvw, f, pc, cfg = sim.observation("small-array", ntimes=1)
    b = sim.make_blockvisibility(uvw, f, pc, cfg)
    b["vis"].data[...] = 1.0
    off = SkyDirection(pc.ra.rad + 0.01, pc.dec.rad - 0.005)
    im = sim.model_image(cfg, sim.sources(cfg), off, f)
    s = shift_vis_to_image(b, im, tangent=True, inverse=False)
    l, m, n = lmn_of(off, pc)
    d = numpy.array([l, m, numpy.sqrt(1 - l * l - m * m) - 1.0])
    ph = numpy.exp(2j * numpy.pi * (uvw @ d)[..., None] * f / 299792458.0)
    numpy.testing.assert_allclose(s["vis"].data[..., 0], ph, rtol=0, atol=1e-12)
    assert s.phasecentre is im.image_acc.phasecentre
    inv = shift_vis_to_image(b, im, tangent=True, inverse=True)
    numpy.testing.assert_allclose(inv["vis"].data[..., 0], numpy.conj(ph), rtol=0, atol=1e-12)
    assert shift_vis_to_image(s, im, tangent=True, inverse=True) is s


def _offset_case(precision, ntimes=16, nchan=3):
    from rascil_gb300 import data_models as dm
    from rascil_gb300 import simulation as sim
    uvw, freq, pc, cfg = sim.observation("small-array", seed=0, ntimes=ntimes, nchan=nchan, npixel=256)
    if len(freq) > 1 and freq[0] == freq[-1]:
        freq = numpy.linspace(1.0e8, 1.2e8, nchan)
    rng = numpy.random.default_rng(7)
    dtype = numpy.complex128 if precision == "fp64" else numpy.complex64
    shape = uvw.shape[:2] + (len(freq), 1)
    vis = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(dtype)
    bvis = sim.make_blockvisibility(uvw, freq, pc, cfg, vis=vis)
    bvis["imaging_weight"].data[...] = rng.uniform(0.5, 1.5, shape)
    off = dm.SkyDirection(pc.ra.rad + 0.004, pc.dec.rad - 0.003)
    empty = ([], [], [], [], [])
    model_off = sim.model_image(cfg, empty, off, freq)
    model_pc = sim.model_image(cfg, empty, pc, freq)
    l, m, n = lmn_of_direction(off.ra.rad, off.dec.rad, pc.ra.rad, pc.dec.rad)
    return uvw, freq, bvis, model_off, model_pc, (l, m, n - 1.0), off


PREC = [("fp64", 1e-12, 1e-12), ("fp32", 1e-5, 1e-5)]


@pytest.mark.parametrize("precision,eps,tol", PREC)
def test_invert_with_offset_image_equals_invert_of_rotated_vis(precision, eps, tol):
    from rascil_gb300.data_models import copy_visibility
    from rascil_gb300.imaging import invert_ng
    uvw, freq, bvis, model_off, model_pc, lmn, off = _offset_case(precision)
    got, sw = invert_ng(bvis, model_off, epsilon=eps, precision=precision)
    vis = bvis["vis"].data.astype(numpy.complex128)
    rotated = copy_visibility(
        bvis, vis=orot.phaserotate(vis, uvw, freq, lmn).astype(bvis["vis"].data.dtype))
    ref, sw_ref = invert_ng(rotated, model_pc, epsilon=eps, precision=precision)
    numpy.testing.assert_allclose(sw, sw_ref, rtol=1e-12)
    assert rel_rms(got["pixels"].data, ref["pixels"].data) < tol
    # the cached shifted plan is not reused for the centred image
    again, _ = invert_ng(bvis, model_pc, epsilon=eps, precision=precision)
    assert rel_rms(again["pixels"].data, got["pixels"].data) > 1e-3


@pytest.mark.parametrize("precision,eps,tol", [("fp64", 1e-12, 1e-12), ("fp32", 1e-5, 1e-6)])
def test_psf_of_offset_image_ignores_the_shift(precision, eps, tol):
    from rascil_gb300.imaging import invert_ng
    _, _, bvis, model_off, model_pc, _, _ = _offset_case(precision)
    got, sw = invert_ng(bvis, model_off, dopsf=True, epsilon=eps, precision=precision)
    ref, sw_ref = invert_ng(bvis, model_pc, dopsf=True, epsilon=eps, precision=precision)
    numpy.testing.assert_allclose(sw, sw_ref, rtol=1e-12)
    assert rel_rms(got["pixels"].data, ref["pixels"].data) < tol
    assert abs(float(numpy.max(got["pixels"].data)) - 1.0) < 10 * tol


@pytest.mark.parametrize("precision,eps,tol", PREC)
def test_predict_with_offset_image_equals_rotated_prediction(precision, eps, tol):
    from rascil_gb300.imaging import predict_ng
    uvw, freq, bvis, model_off, model_pc, lmn, off = _offset_case(precision)
    rng = numpy.random.default_rng(3)
    pix = numpy.zeros(model_pc["pixels"].data.shape)
    ny, nx = pix.shape[-2:]
    for _ in range(12):
        pix[0, 0, rng.integers(ny // 4, 3 * ny // 4), rng.integers(nx // 4, 3 * nx // 4)] = \
            rng.uniform(0.5, 2.0)
    model_off["pixels"].data[...] = pix
    model_pc["pixels"].data[...] = pix
    got = predict_ng(bvis, model_off, epsilon=eps, precision=precision)
    centred = predict_ng(bvis, model_pc, epsilon=eps, precision=precision)["vis"].data
    ref = orot.phaserotate(centred.astype(numpy.complex128), uvw, freq, lmn, inverse=True)
    assert rel_rms(got["vis"].data, ref) < tol
    assert got.phasecentre is model_off.image_acc.phasecentre
    assert bvis.phasecentre is not model_off.image_acc.phasecentre
