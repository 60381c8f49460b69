"""GPU parity of the gridder against the FP64 oracle (exact DFT) and the
CPU restatement of the bucket sort.  Tolerances: FP64 form at
epsilon=1e-12 within 1e-10 relative RMS; FP32 form at epsilon=1e-5
within 1e-5 relative RMS (both against the exact direct sum)."""
import numpy
import pytest

from oracle import dft
from oracle import wgridder as owg
from tests.cases import random_problem, rel_rms

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FORMS = [("fp64", 1e-12, 1e-10), ("fp32", 1e-5, 1e-5)]


def _dev(x, dtype):
    return torch.from_numpy(numpy.ascontiguousarray(x)).to("cuda", dtype)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("do_w", [False, True])
def test_bucket_keys_bit_exact(precision, do_w):
    from rascil_gb300 import wgridder, _lib
    import ctypes
    c = random_problem(seed=3, nrow=1500, nchan=4, uvscale=9000.0)
    eps = 1e-12 if precision == "fp64" else 1e-5
    uvw = _dev(c["uvw"], torch.float64)
    freq = _dev(c["freq"], torch.float64)
    plan = wgridder.Plan(uvw, freq, c["npix"], c["npix"], c["pixsize"], c["pixsize"], eps,
                         do_w, precision=precision)
    info = plan.info
    n = plan.nrows * plan.nchan
    bucket = torch.empty(n, dtype=torch.int32, device="cuda")
    cell = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    frac = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    _lib.check(_lib.load().gb_plan_export_items(plan._handle, ctypes.c_void_p(bucket.data_ptr()),
                                                ctypes.c_void_p(cell.data_ptr()),
                                                ctypes.c_void_p(frac.data_ptr()),
                                                wgridder._stream(uvw.device)))
    torch.cuda.synchronize()
    s = c["freq"] / dft.SPEED_OF_LIGHT
    w_all = c["uvw"][:, 2:3] * s
    op = owg.Plan(c["npix"], c["npix"], c["pixsize"], c["pixsize"], eps, do_w,
                  *owg.w_range(w_all, do_w), fp32=precision == "fp32")
    assert (op.W, op.ngx, op.nplanes) == (info["support"], info["ngrid_x"], info["nplanes"])
    assert op.dw == info["dw"] and op.tc == info["tc"]
    p0, q0, k0, du, dv, dwf, _, flip = (x.ravel() for x in op.coords(c["uvw"], c["freq"]))
    assert flip.any() == do_w  # with w-stacking the rows with w < 0 are mirrored
    cell = cell.cpu().numpy()
    numpy.testing.assert_array_equal(cell[:, 0], p0)
    numpy.testing.assert_array_equal(cell[:, 1], q0)
    numpy.testing.assert_array_equal(cell[:, 2], k0)
    T, S = info["tile"], info["slab"]
    ntu = -(-op.ngx // T)
    ntv = -(-op.ngy // T)
    key = ((k0 // S) * ntv + q0 // T) * ntu + p0 // T
    numpy.testing.assert_array_equal(bucket.cpu().numpy().astype(numpy.int64), key)
    frac = frac.cpu().numpy()
    if precision == "fp64":
        numpy.testing.assert_array_equal(frac[:, 0], du)
        numpy.testing.assert_array_equal(frac[:, 1], dv)
        if do_w:
            numpy.testing.assert_array_equal(frac[:, 2], dwf)
    else:
        numpy.testing.assert_array_equal(frac[:, 0], du.astype(numpy.float32))
        numpy.testing.assert_array_equal(frac[:, 1], dv.astype(numpy.float32))
    plan.close()


@pytest.mark.parametrize("precision,eps,tol", FORMS)
@pytest.mark.parametrize("do_w", [False, True])
def test_ms2dirty_matches_dft(precision, eps, tol, do_w):
    from rascil_gb300 import wgridder
    c = random_problem(seed=1)
    ms = c["ms"][..., 0]
    wgt = c["wgt"][..., 0]
    ref = dft.ms2dirty_dft(c["uvw"], c["freq"], ms, wgt, c["npix"], c["npix"], c["pixsize"],
                           c["pixsize"], do_w)
    cdt = numpy.complex128 if precision == "fp64" else numpy.complex64
    rdt = numpy.float64 if precision == "fp64" else numpy.float32
    got = wgridder.ms2dirty(c["uvw"], c["freq"], ms.astype(cdt), wgt.astype(rdt), c["npix"],
                            c["npix"], c["pixsize"], c["pixsize"], 0, 0, eps, do_w)
    assert got.shape == (c["npix"], c["npix"])
    assert rel_rms(got, ref) < tol


@pytest.mark.parametrize("precision,eps,tol", FORMS)
@pytest.mark.parametrize("do_w", [False, True])
def test_dirty2ms_matches_dft(precision, eps, tol, do_w):
    from rascil_gb300 import wgridder
    c = random_problem(seed=2)
    img = c["img"][0]
    ref = dft.dirty2ms_dft(c["uvw"], c["freq"], img, None, c["pixsize"], c["pixsize"], do_w)
    rdt = numpy.float64 if precision == "fp64" else numpy.float32
    got = wgridder.dirty2ms(c["uvw"], c["freq"], img.astype(rdt), None, c["pixsize"],
                            c["pixsize"], 0, 0, eps, do_w)
    assert got.shape == ref.shape
    assert rel_rms(got, ref) < tol


@pytest.mark.parametrize("precision,eps,tol", FORMS)
def test_adjointness(precision, eps, tol):
    """<A^H v, x> == Re <v, A x> for the plan's invert/predict pair."""
    from rascil_gb300 import wgridder
    c = random_problem(seed=4)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    rdt = torch.float64 if precision == "fp64" else torch.float32
    plan = wgridder.Plan(_dev(c["uvw"], torch.float64), _dev(c["freq"], torch.float64),
                         c["npix"], c["npix"], c["pixsize"], c["pixsize"], eps, True,
                         precision=precision)
    v = _dev(c["ms"], cdt)
    x = _dev(c["img"], rdt)
    aht_v = plan.ms2dirty(v).double().cpu().numpy()
    a_x = plan.dirty2ms(x).cpu().numpy().astype(numpy.complex128)
    lhs = float(numpy.sum(aht_v * c["img"]))
    rhs = float(numpy.real(numpy.vdot(a_x, c["ms"])))
    assert abs(lhs - rhs) <= 10 * tol * max(abs(lhs), abs(rhs))
    plan.close()


@pytest.mark.parametrize("precision,eps,tol", FORMS)
def test_four_pols_with_matrix(precision, eps, tol):
    """npol=4 in one pass with a linear->Stokes matrix equals per-pol oracle calls."""
    from rascil_gb300 import wgridder
    c = random_problem(seed=5, npol=4)
    m = numpy.array([[0.5, 0, 0, 0.5], [0.5, 0, 0, -0.5], [0, 0.5, 0.5, 0],
                     [0, -0.5j, 0.5j, 0]], dtype=numpy.complex128)
    conv = numpy.einsum("pq,rcq->rcp", m, c["ms"])
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    rdt = torch.float64 if precision == "fp64" else torch.float32
    plan = wgridder.Plan(_dev(c["uvw"], torch.float64), _dev(c["freq"], torch.float64),
                         c["npix"], c["npix"], c["pixsize"], c["pixsize"], eps, True,
                         npol=4, precision=precision)
    dirty, sw = plan.ms2dirty(_dev(c["ms"], cdt), wgt=_dev(c["wgt"], rdt), polmat=m,
                              layout="yx", sumwt=True)
    dirty = dirty.cpu().numpy()
    for p in range(4):
        ref = dft.ms2dirty_dft(c["uvw"], c["freq"], conv[..., p], c["wgt"][..., p], c["npix"],
                               c["npix"], c["pixsize"], c["pixsize"], True)
        assert rel_rms(dirty[p].T, ref) < tol
    wref = c["wgt"].astype(numpy.float64 if precision == "fp64" else numpy.float32)
    numpy.testing.assert_allclose(sw.cpu().numpy(), wref.astype(numpy.float64).sum(axis=(0, 1)),
                                  rtol=1e-12)
    # predict with the inverse matrix back to the vis frame
    minv = numpy.linalg.inv(m)
    vis = plan.dirty2ms(_dev(c["img"], rdt), polmat=minv, layout="yx").cpu().numpy()
    ref = numpy.stack([dft.dirty2ms_dft(c["uvw"], c["freq"], c["img"][p].T, None, c["pixsize"],
                                        c["pixsize"], True) for p in range(4)], axis=-1)
    ref = numpy.einsum("qp,rcp->rcq", minv, ref)
    assert rel_rms(vis, ref) < tol
    plan.close()
