"""GPU parity of the FP32 column-transform path (fused, pruned four-step
column FFTs with the w-screen folded in; predict grids in permuted row
order).  Small images are checked against the FP64 direct sum (oracle) at
the FP32 bar, 1e-5 relative RMS; tall, ragged, wide-grid and multi-pol
images against the plain FP64 GPU form, which is itself held to 1e-10
against the direct sum, at the same bar, and the tall and wide-grid ones
also against the CPU oracle's direct sums at sampled pixels and rows; and
the two FP32 modes against each other."""
import numpy
import pytest

from oracle import dft
from tests.cases import random_problem, rel_rms

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5


def _dev(x, dtype):
    return torch.from_numpy(numpy.ascontiguousarray(x)).to("cuda", dtype)


def _check_oracle_samples(c, nx, ny, dirty, img, vis, nsample=64, seed=99):
    """An FP32 dirty image ([1][x][y]) and prediction ([nrow][nchan][1]) of
    the Stokes-I problem `c` against the CPU oracle's exact direct sums at
    `nsample` random pixels and rows, at the FP32 bar."""
    rng = numpy.random.default_rng(seed)
    ix = rng.integers(0, nx, nsample)
    iy = rng.integers(0, ny, nsample)
    ref = dft.ms2dirty_dft(c["uvw"], c["freq"], c["ms"][..., 0], None, nx, ny, c["pixsize"],
                           c["pixsize"], True, pixel_subset=(ix, iy))
    assert rel_rms(dirty[0, ix, iy], ref) < TOL
    rows = numpy.sort(rng.choice(c["uvw"].shape[0], nsample, replace=False))
    vref = dft.dirty2ms_dft(c["uvw"], c["freq"], img[0], None, c["pixsize"], c["pixsize"], True,
                            row_subset=rows, chunk=16)
    assert rel_rms(vis[rows, :, 0], vref) < TOL


def _plan(c, nx, ny, do_w, precision, fft_mode, npol=1, eps=1e-5, **kw):
    from rascil_gb300 import wgridder
    return wgridder.Plan(_dev(c["uvw"], torch.float64), _dev(c["freq"], torch.float64), nx, ny,
                         c["pixsize"], c["pixsize"], eps, do_w, npol=npol, precision=precision,
                         fft_mode=fft_mode, sigma=2.0, **kw)


def test_mode_selection():
    """auto picks the column kernels only for the FP32 form with a
    power-of-two grid height; asking for them elsewhere is an error."""
    c = random_problem(seed=11, nrow=50, nchan=1, npix=128)
    p = _plan(c, 128, 128, True, "fp32", "auto")
    assert p.info["ngrid_y"] == 256 and p.info["fft_mode"] == 2
    p.close()
    p = _plan(c, 128, 128, True, "fp64", "auto")
    assert p.info["fft_mode"] == 1
    p.close()
    p = _plan(c, 128, 128, True, "fp32", "cufft2d")
    assert p.info["fft_mode"] == 1
    p.close()
    with pytest.raises(ValueError, match="GB_FFT_COLUMNS"):
        _plan(c, 96, 96, True, "fp32", "columns")  # grid 192
    with pytest.raises(ValueError, match="GB_FFT_COLUMNS"):
        _plan(c, 128, 128, True, "fp64", "columns")


@pytest.mark.parametrize("do_w", [False, True])
@pytest.mark.parametrize("nx,ny", [(128, 128), (200, 256), (256, 128)])
def test_invert_predict_vs_dft(do_w, nx, ny):
    c = random_problem(seed=21, nrow=300, nchan=3, npix=max(nx, ny), pixsize=1.5e-3,
                       uvscale=4000.0)
    ms = c["ms"][..., 0]
    wgt = c["wgt"][..., 0]
    p = _plan(c, nx, ny, do_w, "fp32", "columns")
    assert p.info["fft_mode"] == 2
    dirty = p.ms2dirty(_dev(ms[..., None], torch.complex64), wgt=_dev(wgt[..., None],
                                                                       torch.float32),
                       layout="xy")[0].double().cpu().numpy()
    ref = dft.ms2dirty_dft(c["uvw"], c["freq"], ms, wgt, nx, ny, c["pixsize"], c["pixsize"], do_w)
    assert rel_rms(dirty, ref) < TOL
    rng = numpy.random.default_rng(5)
    img = rng.normal(size=(nx, ny))
    vis = p.dirty2ms(_dev(img[None], torch.float32), layout="xy")[..., 0].cpu().numpy()
    vref = dft.dirty2ms_dft(c["uvw"], c["freq"], img, None, c["pixsize"], c["pixsize"], do_w)
    assert rel_rms(vis, vref) < TOL
    assert p.device_status() == 0
    p.close()


# (nx, ny): grid heights 512 .. 32768 cover every column split N1 x N2
# (16x32, 32x32, 32x64, 64x64, 64x128, 128x128, 128x256); odd widths leave
# a ragged last column tile.
SHAPES = [(200, 256), (56, 512), (96, 1024), (72, 2048), (64, 4096), (48, 8192), (40, 16384)]


@pytest.mark.parametrize("nx,ny", SHAPES)
def test_tall_images_vs_fp64(nx, ny):
    c = random_problem(seed=31, nrow=2000, nchan=2, npix=8, pixsize=5e-5, uvscale=30000.0,
                       wscale=3000.0)
    pf = _plan(c, nx, ny, True, "fp32", "columns")
    pd = _plan(c, nx, ny, True, "fp64", "auto", eps=1e-12)
    assert pf.info["fft_mode"] == 2
    vis = c["ms"]
    dirty32 = pf.ms2dirty(_dev(vis, torch.complex64)).double().cpu().numpy()
    dirty64 = pd.ms2dirty(_dev(vis, torch.complex128)).cpu().numpy()
    assert rel_rms(dirty32, dirty64) < TOL
    rng = numpy.random.default_rng(7)
    img = rng.normal(size=(1, nx, ny))
    v32 = pf.dirty2ms(_dev(img, torch.float32)).cpu().numpy()
    v64 = pd.dirty2ms(_dev(img, torch.float64)).cpu().numpy()
    assert rel_rms(v32, v64) < TOL
    _check_oracle_samples(c, nx, ny, dirty32, img, v32)
    assert pf.device_status() == 0
    pf.close()
    pd.close()


@pytest.mark.parametrize("npol", [2, 4])
def test_multi_pol_and_batches(npol):
    """Several polarisations and several plane batches (small grid budget),
    so step B accumulates across batches and predict rows are permuted in
    every batch."""
    c = random_problem(seed=41, nrow=1500, nchan=3, npix=512, pixsize=4e-4, uvscale=20000.0,
                       wscale=6000.0, npol=npol)
    kw = dict(grid_budget_bytes=3 * npol * 1024 * 1024 * 8)
    pc = _plan(c, 512, 512, True, "fp32", "columns", npol=npol, **kw)
    pd = _plan(c, 512, 512, True, "fp64", "auto", npol=npol, eps=1e-12, **kw)
    assert pc.info["planes_per_batch"] < pc.info["nplanes"]
    d32 = pc.ms2dirty(_dev(c["ms"], torch.complex64), wgt=_dev(c["wgt"], torch.float32))
    d64 = pd.ms2dirty(_dev(c["ms"], torch.complex128), wgt=_dev(c["wgt"], torch.float64))
    assert rel_rms(d32.double().cpu().numpy(), d64.cpu().numpy()) < TOL
    v32 = pc.dirty2ms(_dev(c["img"], torch.float32)).cpu().numpy()
    v64 = pd.dirty2ms(_dev(c["img"], torch.float64)).cpu().numpy()
    assert rel_rms(v32, v64) < TOL
    assert pc.device_status() == 0
    pc.close()
    pd.close()


def test_modes_agree():
    """The column path and the 2-D cuFFT path of the FP32 form agree far
    below the FP32 bar."""
    c = random_problem(seed=51, nrow=2000, nchan=4, npix=1024, pixsize=1e-4, uvscale=40000.0,
                       wscale=8000.0)
    a = _plan(c, 1024, 1024, True, "fp32", "columns")
    b = _plan(c, 1024, 1024, True, "fp32", "cufft2d")
    va = _dev(c["ms"], torch.complex64)
    da = a.ms2dirty(va).double().cpu().numpy()
    db = b.ms2dirty(va).double().cpu().numpy()
    assert rel_rms(da, db) < 2e-6
    img = _dev(c["img"], torch.float32)
    assert rel_rms(a.dirty2ms(img).cpu().numpy(), b.dirty2ms(img).cpu().numpy()) < 2e-6
    assert a.device_status() == 0
    a.close()
    b.close()


# (nx, ny): grid widths 4096, 8192, 16384 run the library's row kernels
# (k_rows, one CTA per row, empty rows skipped); short images keep it cheap.
WIDE = [(2048, 128), (4096, 256), (8192, 128)]


@pytest.mark.parametrize("nx,ny", WIDE)
def test_row_kernel_vs_fp64(nx, ny):
    c = random_problem(seed=61, nrow=3000, nchan=2, npix=8, pixsize=5e-5, uvscale=30000.0,
                       wscale=3000.0)
    pf = _plan(c, nx, ny, True, "fp32", "columns")
    pd = _plan(c, nx, ny, True, "fp64", "auto", eps=1e-12)
    assert pf.info["fft_mode"] == 2 and pf.info["own_rows"] == 1
    vis = c["ms"]
    d32 = pf.ms2dirty(_dev(vis, torch.complex64)).double().cpu().numpy()
    d64 = pd.ms2dirty(_dev(vis, torch.complex128)).cpu().numpy()
    assert rel_rms(d32, d64) < TOL
    rng = numpy.random.default_rng(8)
    img = rng.normal(size=(1, nx, ny))
    v32 = pf.dirty2ms(_dev(img, torch.float32)).cpu().numpy()
    v64 = pd.dirty2ms(_dev(img, torch.float64)).cpu().numpy()
    assert rel_rms(v32, v64) < TOL
    _check_oracle_samples(c, nx, ny, d32, img, v32)
    assert pf.device_status() == 0
    pf.close()
    pd.close()


def test_row_kernel_vs_dft():
    """Own rows against the direct sum, 4 pols, several plane batches."""
    nx, ny = 2048, 128
    c = random_problem(seed=62, nrow=200, nchan=2, npix=8, pixsize=1e-4, uvscale=8000.0,
                       wscale=2000.0, npol=4)
    p = _plan(c, nx, ny, True, "fp32", "columns", npol=4,
              grid_budget_bytes=2 * 4 * 4096 * 256 * 8)
    assert p.info["own_rows"] == 1 and p.info["planes_per_batch"] < p.info["nplanes"]
    dirty = p.ms2dirty(_dev(c["ms"], torch.complex64), wgt=_dev(c["wgt"], torch.float32),
                       layout="xy").double().cpu().numpy()
    for q in (0, 3):
        ref = dft.ms2dirty_dft(c["uvw"], c["freq"], c["ms"][..., q], c["wgt"][..., q], nx, ny,
                               c["pixsize"], c["pixsize"], True)
        assert rel_rms(dirty[q], ref) < TOL
    rng = numpy.random.default_rng(9)
    img = rng.normal(size=(4, nx, ny))
    vis = p.dirty2ms(_dev(img, torch.float32), layout="xy").cpu().numpy()
    for q in (1, 2):
        vref = dft.dirty2ms_dft(c["uvw"], c["freq"], img[q], None, c["pixsize"], c["pixsize"],
                                True)
        assert rel_rms(vis[..., q], vref) < TOL
    assert p.device_status() == 0
    p.close()
