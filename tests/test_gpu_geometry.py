"""GPU parity at the benchmark geometries, against the CPU oracle.

The headline workload images LOW-like geometry (512 stations to 35 km, dec
-30 deg, 100-200 MHz) and the stress configuration MID-like geometry (197
dishes to 80 km, dec -60 deg, 0.95-1.67 GHz).  There the FP64 phase
wrap of u dx and the fixed-point w-screen turns are stressed hardest.  These
tests keep every baseline, the band edges and the declination, with few
times and channels, and check both forms against the oracle's FP64 direct
sums (``oracle/dft.py``: the exact operators ducc0.wgridder approximates,
called by ``rascil/processing_components/imaging/ng.py:91-103,232-248``)
at sampled pixels (invert) and rows (predict):

* FP32 form at epsilon 1e-5: relative RMS <= 1e-5;
* FP64 form at epsilon 1e-12: relative RMS <= 1e-10.

The wide-grid cases (grids of 8192 and 16384 cells, the library's own row
and column transforms that the headline step runs) are checked the same
way.  The truth is always the CPU oracle, never a GPU kernel.
"""
import numpy
import pytest

from oracle import dft as odft
from tests.cases import rel_rms

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _geometry(name, ntimes, nchan, npixel, cell, nsrc=40, seed=0):
    """Flipped uvw (as ng.py passes them), freq (band edges), a sparse model
    image [x][y] of point sources and visibilities of those sources."""
    from rascil_gb300 import simulation as sim
    uvw, freq, pc, cfg = sim.observation(name, seed=seed, ntimes=ntimes, nchan=nchan,
                                         npixel=npixel)
    cfg = dict(cfg, nsrc=nsrc, cellsize=cell)
    ix, iy, l, m, flux = sim.sources(cfg, seed=seed)
    fu = uvw.reshape(-1, 3) * numpy.array([-1.0, 1.0, -1.0])
    # pixel-centre sources: the exact image-plane operator gives their
    # visibilities (and the model image for predict)
    dirty = numpy.zeros((npixel, npixel))
    numpy.add.at(dirty, (ix, iy), flux)
    return fu, freq, dirty, (ix, iy)


def _check(fu, freq, dirty, src_pix, npix, cell, precision, eps, tol, fft_expect=None,
           nrows_check=192, npix_check=48, sigma=0.0):
    from rascil_gb300.wgridder import Plan
    rng = numpy.random.default_rng(11)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    rdt = torch.float64 if precision == "fp64" else torch.float32
    u = torch.from_numpy(fu.copy()).cuda()
    f = torch.from_numpy(freq.copy()).cuda()
    plan = Plan(u, f, npix, npix, cell, cell, eps, True, npol=1, precision=precision,
                sigma=sigma)
    try:
        if fft_expect is not None:
            assert (plan.info["fft_mode"], plan.info["own_rows"]) == fft_expect, plan.info
        # predict: model image -> visibilities at sampled rows
        model = torch.from_numpy(dirty).to(device="cuda", dtype=rdt).reshape(1, npix, npix)
        pred = plan.dirty2ms(model, layout="xy")
        rows = numpy.sort(rng.choice(fu.shape[0], min(nrows_check, fu.shape[0]), replace=False))
        got_v = pred[torch.from_numpy(rows).cuda(), :, 0].to(torch.complex128).cpu().numpy()
        truth_v = odft.dirty2ms_dft(fu, freq, dirty, None, cell, cell, True, row_subset=rows)
        e_pred = rel_rms(got_v, truth_v)
        # invert: the model's exact visibilities (CPU oracle, FP64) -> dirty
        # image at the sources' pixels and at random pixels
        vis = odft.dirty2ms_dft(fu, freq, dirty, None, cell, cell, True)
        img = plan.ms2dirty(torch.from_numpy(vis).to(device="cuda", dtype=cdt)
                            .reshape(plan.nrows, plan.nchan, 1), layout="xy")[0]
        k = npix_check // 2
        pix = numpy.concatenate([numpy.stack(src_pix, -1)[:k],
                                 rng.integers(0, npix, (k, 2))])
        got_px = img.double().cpu().numpy()[pix[:, 0], pix[:, 1]]
        truth_px = odft.ms2dirty_dft(fu, freq, vis, None, npix, npix, cell, cell, True,
                                     pixel_subset=(pix[:, 0], pix[:, 1]), chunk=8)
        e_inv = rel_rms(got_px, truth_px)
        assert e_pred <= tol, ("predict", precision, e_pred, plan.info)
        assert e_inv <= tol, ("invert", precision, e_inv, plan.info)
        return plan.info
    finally:
        plan.close()


FORMS = [("fp32", 1e-5, 1e-5), ("fp64", 1e-12, 1e-10)]


@pytest.mark.parametrize("precision,eps,tol", FORMS)
def test_low_like_geometry_against_cpu_oracle(precision, eps, tol):
    """Every LOW-like baseline (to 35 km), 2 times, 100 and 200 MHz, 1024^2
    at the configured 1e-5 rad cell."""
    fu, freq, dirty, src = _geometry("low-like", 2, 2, 1024, 1e-5)
    _check(fu, freq, dirty, src, 1024, 1e-5, precision, eps, tol)


@pytest.mark.parametrize("cell", [5e-7, 2e-5])
@pytest.mark.parametrize("precision,eps,tol", FORMS)
def test_mid_like_geometry_against_cpu_oracle(precision, eps, tol, cell):
    """Every MID-like baseline (to 80 km), 2 times, 0.95 and 1.67 GHz, 1024^2:
    at the configured 5e-7 rad cell (u dx reaches ~220 turns, wrapped in
    FP64) and at 2e-5 rad (a wider field: w to 4.5e5 wavelengths over many
    w-planes, screen phases of tens of turns)."""
    fu, freq, dirty, src = _geometry("mid-like", 2, 2, 1024, cell)
    info = _check(fu, freq, dirty, src, 1024, cell, precision, eps, tol)
    if cell > 1e-6:
        assert info["nplanes"] > 2 * info["support"]  # the w-stacking is exercised


@pytest.mark.parametrize("npix,own_rows", [(4096, 1), (8192, 1)])
def test_wide_grid_column_mode_against_cpu_oracle(npix, own_rows):
    """FP32 form with the library's own row and column transforms on grids
    of 8192 and 16384 cells (the headline's transforms), LOW-like baselines."""
    fu, freq, dirty, src = _geometry("low-like", 1, 2, npix, 1e-5)
    _check(fu, freq, dirty, src, npix, 1e-5, "fp32", 1e-5, 1e-5, fft_expect=(2, own_rows),
           nrows_check=128, npix_check=32, sigma=2.0)


@pytest.mark.parametrize("precision,eps,tol,sigma", [("fp32", 1e-5, 1e-5, 1.5),
                                                      ("fp32", 1e-5, 1e-5, 1.75),
                                                      ("fp64", 1e-12, 1e-10, 1.25),
                                                      ("fp64", 1e-8, 1e-7, 1.25)])
def test_low_like_geometry_other_oversampling(precision, eps, tol, sigma):
    """Both forms at the other tabulated grid oversamplings (batched cuFFT
    transforms, larger supports, the w-screen phases in fixed point),
    LOW-like baselines."""
    fu, freq, dirty, src = _geometry("low-like", 2, 2, 1024, 1e-5)
    try:
        info = _check(fu, freq, dirty, src, 1024, 1e-5, precision, eps, tol, sigma=sigma)
    except ValueError as e:  # epsilon out of this oversampling's reach
        assert precision == "fp64" and eps == 1e-12 and "not reachable" in str(e)
        return
    assert info["sigma"] == sigma and info["fft_mode"] == 1


def test_fp32_form_refuses_sigma_125():
    """At sigma 1.25 the edge correction amplifies FP32 grid rounding beyond
    epsilon 1e-5, so the FP32 form refuses it (and the planner never picks it)."""
    from rascil_gb300.wgridder import Plan
    fu, freq, dirty, src = _geometry("low-like", 1, 1, 256, 1e-5)
    u = torch.from_numpy(fu.copy()).cuda()
    f = torch.from_numpy(freq.copy()).cuda()
    with pytest.raises(ValueError, match="sigma >= 1.5"):
        Plan(u, f, 256, 256, 1e-5, 1e-5, 1e-5, True, precision="fp32", sigma=1.25)
