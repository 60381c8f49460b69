"""GPU parity of the list workflows (rascil_gb300/workflows.py) with the
reference's composition of the single-block functions
(rascil/workflows/rsexecute/imaging/imaging_rsexecute.py:72-181,913-930,
rascil/processing_components/imaging/imaging_helpers.py:17-42):

* blocks run concurrently on several streams give the results of running
  invert_ng / predict_ng on each block in turn;
* the fused residual equals predict -> subtract -> invert composed from the
  list functions, also with a model centred away from the phase centre;
* sum_invert_results reproduces the reference's known answers
  (tests/workflows/test_sum_invert_rsexecute.py: ten constant images i+1
  with weights i+1 sum to 7 everywhere), and summing the inverts of time
  blocks equals the invert of all the rows at once.

Tolerances: FP64 form 1e-12 relative RMS (only summation order differs);
FP32 form 1e-5 (its accuracy bar).
"""
import numpy
import pytest

from tests.cases import rel_rms

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _time_blocks(precision, splits=(3, 5, 8), npixel=256, seed=1):
    """One small-array observation cut into uneven time blocks, random vis and
    weights, flags on 5 %."""
    from rascil_gb300 import simulation as sim
    uvw, freq, pc, cfg = sim.observation("small-array", seed=0, ntimes=sum(splits), npixel=npixel)
    rng = numpy.random.default_rng(seed)
    dtype = numpy.complex128 if precision == "fp64" else numpy.complex64
    shape = uvw.shape[:2] + (len(freq), 1)
    vis = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(dtype)
    whole = sim.make_blockvisibility(uvw, freq, pc, cfg, vis=vis)
    whole["imaging_weight"].data[...] = rng.uniform(0.5, 1.5, shape)
    whole["flags"].data[...] = (rng.uniform(size=shape) < 0.05).astype(numpy.int64)
    blocks, t0 = [], 0
    for n in splits:
        b = sim.make_blockvisibility(uvw[t0:t0 + n], freq, pc, cfg, vis=vis[t0:t0 + n].copy())
        b["imaging_weight"].data[...] = whole["imaging_weight"].data[t0:t0 + n]
        b["flags"].data[...] = whole["flags"].data[t0:t0 + n]
        blocks.append(b)
        t0 += n
    model = sim.model_image(cfg, ([], [], [], [], []), pc, freq)
    return whole, blocks, model, cfg, pc, freq


PREC = [("fp64", 1e-12, 1e-12), ("fp32", 1e-5, 1e-5)]


@pytest.mark.parametrize("precision,eps,tol", PREC)
def test_invert_list_matches_blocks_one_by_one(precision, eps, tol):
    from rascil_gb300 import simulation as sim
    from rascil_gb300.imaging import invert_ng
    from rascil_gb300.workflows import invert_list_rsexecute_workflow
    whole, blocks, model, cfg, pc, freq = _time_blocks(precision)
    # uneven templates: the last block images at 128 pixels
    cfg128 = dict(cfg, npixel=128)
    templates = [model, model, sim.model_image(cfg128, ([], [], [], [], []), pc, freq)]
    kw = dict(epsilon=eps, precision=precision)
    got = invert_list_rsexecute_workflow(blocks, templates, "ng", streams=3, **kw)
    for (im, sw), b, t in zip(got, blocks, templates):
        ref, sw_ref = invert_ng(b, t, **kw)
        numpy.testing.assert_allclose(sw, sw_ref, rtol=1e-12)
        assert rel_rms(im["pixels"].data, ref["pixels"].data) < tol
    psf = invert_list_rsexecute_workflow(blocks, templates, "ng", dopsf=True, streams=3, **kw)
    for im, _ in psf:
        assert abs(float(im["pixels"].data.max()) - 1.0) < 1e-5


@pytest.mark.parametrize("precision,eps,tol", PREC)
def test_predict_list_matches_blocks_and_zeroes_inputs(precision, eps, tol):
    from rascil_gb300.imaging import predict_ng
    from rascil_gb300.workflows import predict_list_rsexecute_workflow, zero_list_rsexecute_workflow
    whole, blocks, model, cfg, pc, freq = _time_blocks(precision)
    rng = numpy.random.default_rng(4)
    ny, nx = model["pixels"].data.shape[-2:]
    for _ in range(10):
        model["pixels"].data[0, 0, rng.integers(ny // 4, 3 * ny // 4),
                             rng.integers(nx // 4, 3 * nx // 4)] = rng.uniform(0.5, 2.0)
    kw = dict(epsilon=eps, precision=precision)
    ref = [predict_ng(b, model, **kw)["vis"].data for b in blocks]
    got = predict_list_rsexecute_workflow(zero_list_rsexecute_workflow(blocks),
                                          [model] * len(blocks), "ng", streams=3, **kw)
    for g, r in zip(got, ref):
        assert rel_rms(g["vis"].data, r) < tol
    # the reference zeroes the blocks it is given, in place
    predict_list_rsexecute_workflow(blocks, [model] * len(blocks), "ng", streams=3, **kw)
    assert all(numpy.all(b["vis"].data == 0) for b in blocks)


@pytest.mark.parametrize("precision,eps,tol", PREC)
@pytest.mark.parametrize("offset", [False, True])
def test_residual_list_matches_composed_workflow(precision, eps, tol, offset):
    """residual_list (fused) == invert_list(subtract_list(vis, predict_list(
    zero_list(vis), models))) run block by block."""
    from rascil_gb300 import simulation as sim
    from rascil_gb300.data_models import SkyDirection, copy_visibility
    from rascil_gb300.workflows import (invert_list_rsexecute_workflow,
                                        predict_list_rsexecute_workflow,
                                        residual_list_rsexecute_workflow,
                                        subtract_list_rsexecute_workflow,
                                        zero_list_rsexecute_workflow)
    whole, blocks, model, cfg, pc, freq = _time_blocks(precision)
    if offset:
        model = sim.model_image(cfg, ([], [], [], [], []),
                                SkyDirection(pc.ra.rad + 0.003, pc.dec.rad + 0.002), freq)
    rng = numpy.random.default_rng(9)
    ny, nx = model["pixels"].data.shape[-2:]
    for _ in range(10):
        model["pixels"].data[0, 0, rng.integers(ny // 4, 3 * ny // 4),
                             rng.integers(nx // 4, 3 * nx // 4)] = rng.uniform(0.5, 2.0)
    models = [model] * len(blocks)
    kw = dict(epsilon=eps, precision=precision)
    got = residual_list_rsexecute_workflow(blocks, models, context="ng", streams=3, **kw)
    mv = predict_list_rsexecute_workflow(zero_list_rsexecute_workflow(blocks), models, "ng",
                                         streams=1, **kw)
    ref = invert_list_rsexecute_workflow(subtract_list_rsexecute_workflow(blocks, mv), models,
                                         "ng", streams=1, **kw)
    for (im, sw), (rim, rsw) in zip(got, ref):
        numpy.testing.assert_allclose(sw, rsw, rtol=1e-12)
        assert rel_rms(im["pixels"].data, rim["pixels"].data) < tol


def test_sum_invert_results_known_answers():
    from rascil_gb300 import data_models as dm
    from rascil_gb300.workflows import sum_invert_results, sum_invert_results_rsexecute
    freq = numpy.linspace(1e8, 1.5e8, 3)
    pc = dm.SkyDirection(numpy.radians(15.0), numpy.radians(-35.0))
    base = dm.create_image(256, 1e-3, pc, frequency=freq)
    nchan, npol = base["pixels"].data.shape[:2]
    results = []
    for i in range(10):
        im = base.copy(deep=True)
        im["pixels"].data[...] = i + 1
        results.append((im, (i + 1) * numpy.ones([nchan, npol])))
    for im, sw in (sum_invert_results(results), sum_invert_results_rsexecute(results)):
        d = im["pixels"].data
        assert numpy.max(d) == pytest.approx(7.0, abs=1e-12)
        assert numpy.min(d) == pytest.approx(7.0, abs=1e-12)
        assert numpy.sum(d) == pytest.approx(1376256.0, rel=1e-12)
        numpy.testing.assert_array_equal(sw, 55.0)
    one = base.copy(deep=True)
    one["pixels"].data[...] = 1
    im, sw = sum_invert_results([(one, numpy.ones([nchan, npol]))])
    assert im is not one and numpy.sum(im["pixels"].data) == 196608.0
    # a channel whose summed weight is zero is zeroed, as normalise_sumwt does
    w0 = numpy.ones([nchan, npol])
    w0[1] = 0.0
    im, sw = sum_invert_results([(one, w0), (one, w0)])
    assert numpy.all(im["pixels"].data[1] == 0) and numpy.all(im["pixels"].data[0] == 1)


@pytest.mark.parametrize("precision,eps,tol", PREC)
def test_sum_of_block_inverts_equals_invert_of_all_rows(precision, eps, tol):
    from rascil_gb300.imaging import invert_ng
    from rascil_gb300.workflows import invert_list_rsexecute_workflow, sum_invert_results
    whole, blocks, model, cfg, pc, freq = _time_blocks(precision)
    kw = dict(epsilon=eps, precision=precision)
    im, sw = sum_invert_results(
        invert_list_rsexecute_workflow(blocks, [model] * len(blocks), "ng", streams=3, **kw))
    ref, sw_ref = invert_ng(whole, model, **kw)
    numpy.testing.assert_allclose(sw, sw_ref, rtol=1e-12)
    assert rel_rms(im["pixels"].data, ref["pixels"].data) < tol


def test_list_program_matches_worker_thread_map():
    """invert_list / predict_list as one device program (gb_batch_run_items:
    per round, every slot's block gridded or degridded in one persistent
    launch) give the worker-thread map's results, with linear -> IQUV
    polarisation matrices, flags, imaging weights and an image centred away
    from the phase centre (the rotation fused into each block's plan)."""
    from rascil_gb300 import simulation as sim
    from rascil_gb300.data_models import SkyDirection, copy_visibility
    from rascil_gb300.workflows import (invert_list_rsexecute_workflow,
                                        predict_list_rsexecute_workflow)
    uvw, freq, pc, cfg = sim.observation("small-array", seed=0, ntimes=12, npixel=128)
    cfg = dict(cfg, pol="linear", image_pol="stokesIQUV")
    rng = numpy.random.default_rng(6)
    blocks = []
    for t0, n in ((0, 3), (3, 4), (7, 5)):
        shape = (n, uvw.shape[1], len(freq), 4)
        vis = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(numpy.complex64)
        b = sim.make_blockvisibility(uvw[t0:t0 + n], freq, pc, cfg, vis=vis)
        b["imaging_weight"].data[...] = rng.uniform(0.5, 1.5, shape)
        b["flags"].data[...] = (rng.uniform(size=shape) < 0.05).astype(numpy.int64)
        blocks.append(b)
    off = SkyDirection(pc.ra.rad + 0.002, pc.dec.rad - 0.001)
    models = [sim.model_image(cfg, ([], [], [], [], []), off, freq) for _ in blocks]
    for m in models:
        m["pixels"].data[0, :, 60:64, 70:72] = rng.uniform(0.5, 1.0, (4, 4, 2))
    kw = dict(epsilon=1e-5, precision="fp32", streams=2)
    a = invert_list_rsexecute_workflow(blocks, models, "ng", program=True, **kw)
    b = invert_list_rsexecute_workflow(blocks, models, "ng", program=False, **kw)
    for (ia, sa), (ib, sb) in zip(a, b):
        numpy.testing.assert_allclose(sa, sb, rtol=1e-6)
        assert rel_rms(ia["pixels"].data, ib["pixels"].data) < 1e-5
    pa = predict_list_rsexecute_workflow([copy_visibility(x) for x in blocks], models, "ng",
                                         program=True, **kw)
    pb = predict_list_rsexecute_workflow([copy_visibility(x) for x in blocks], models, "ng",
                                         program=False, **kw)
    for va, vb in zip(pa, pb):
        assert rel_rms(va["vis"].data, vb["vis"].data) < 1e-5
        assert va.phasecentre.ra.rad == vb.phasecentre.ra.rad
