"""Differentiable predict (configuration 4's shape, reduced): the autograd
adjoint against the dot-product identity, central finite differences and
the oracle's exact adjoint; the gain-gradient kernel against PyTorch's own
complex autograd on the same expression."""
import numpy
import pytest

from oracle import dft as odft
from tests.cases import rel_rms

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _case(precision="fp64", nants=24, ntimes=6, nchan=3, npix=96, seed=0):
    from rascil_gb300 import simulation as sim
    from rascil_gb300.wgridder import Plan
    from rascil_gb300.autograd import baseline_antennas
    uvw, freq, pc, cfg = sim.observation("gain-solve", seed=seed, ntimes=ntimes, nchan=nchan,
                                         nants=nants)
    cell = 2.0e-4
    u = torch.from_numpy(uvw.reshape(-1, 3).copy()).cuda()
    fu = u.clone()
    fu[:, 0].neg_()
    fu[:, 2].neg_()
    f = torch.from_numpy(freq.copy()).cuda()
    eps = 1e-12 if precision == "fp64" else 1e-5
    plan = Plan(fu, f, npix, npix, cell, cell, eps, True, npol=1, precision=precision)
    a1, a2 = baseline_antennas(nants, ntimes, "cuda")
    return dict(uvw=uvw, fuvw=fu, freq=freq, plan=plan, a1=a1, a2=a2, npix=npix, cell=cell,
                nants=nants)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_predict_adjoint_dot_product(precision, tol):
    from rascil_gb300.autograd import predict
    c = _case(precision)
    plan = c["plan"]
    rng = numpy.random.default_rng(1)
    x = torch.tensor(rng.normal(size=(1, c["npix"], c["npix"])), dtype=plan.real_dtype,
                     device="cuda", requires_grad=True)
    y = torch.tensor(rng.normal(size=(plan.nrows, plan.nchan, 1))
                     + 1j * rng.normal(size=(plan.nrows, plan.nchan, 1)),
                     dtype=plan.complex_dtype, device="cuda")
    v = predict(x, plan)
    lhs = torch.real(torch.vdot(y.reshape(-1), v.reshape(-1)))  # Re<y, A x>
    lhs.backward()
    rhs = (x.detach() * x.grad).sum()                             # <x, A^H y>
    lhs = float(lhs.detach())
    assert abs(lhs - float(rhs)) <= tol * abs(lhs) * 10
    # the gradient is the gridder applied to y (float atomics: order-dependent rounding)
    ref = plan.ms2dirty(y, layout="yx")
    assert rel_rms(x.grad.cpu().numpy(), ref.cpu().numpy()) < (1e-12 if precision == "fp64"
                                                                else 1e-5)
    plan.close()


def test_image_gradient_matches_exact_adjoint():
    """dL/dx for L = Re<y, A x> equals the oracle's exact ms2dirty of y."""
    from rascil_gb300.autograd import predict
    c = _case("fp64", nants=12, ntimes=4, npix=48)
    plan = c["plan"]
    rng = numpy.random.default_rng(2)
    x = torch.zeros((1, 48, 48), dtype=torch.float64, device="cuda", requires_grad=True)
    y = rng.normal(size=(plan.nrows, plan.nchan)) + 1j * rng.normal(size=(plan.nrows, plan.nchan))
    yt = torch.tensor(y[..., None], dtype=torch.complex128, device="cuda")
    torch.real(torch.vdot(yt.reshape(-1), predict(x, plan).reshape(-1))).backward()
    ref = odft.ms2dirty_dft(c["fuvw"].cpu().numpy(), c["freq"], y, None, 48, 48, c["cell"],
                            c["cell"], True)
    assert rel_rms(x.grad[0].cpu().numpy(), ref.T) < 1e-10
    plan.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gain_gradient_kernel_matches_torch_autograd(precision):
    from rascil_gb300.autograd import apply_gains
    c = _case(precision)
    plan = c["plan"]
    rng = numpy.random.default_rng(3)
    shape = (plan.nrows, plan.nchan, 1)
    vis = torch.tensor(rng.normal(size=shape) + 1j * rng.normal(size=shape),
                       dtype=plan.complex_dtype, device="cuda")
    obs = torch.tensor(rng.normal(size=shape) + 1j * rng.normal(size=shape),
                       dtype=plan.complex_dtype, device="cuda")
    g0 = (1 + 0.05 * rng.normal(size=(c["nants"], plan.nchan))) * numpy.exp(
        1j * rng.uniform(-numpy.pi / 8, numpy.pi / 8, (c["nants"], plan.nchan)))
    g = torch.tensor(g0, dtype=torch.complex128, device="cuda", requires_grad=True)
    loss = (apply_gains(vis, g, c["a1"], c["a2"]) - obs).abs().pow(2).sum()
    loss.backward()
    # PyTorch's own complex autograd on the same expression
    gr = torch.tensor(g0, dtype=torch.complex128, device="cuda", requires_grad=True)
    a1, a2 = c["a1"].long(), c["a2"].long()
    fac = (gr[a1] * gr[a2].conj()).unsqueeze(-1)
    lr = (fac * vis.to(torch.complex128) - obs.to(torch.complex128)).abs().pow(2).sum()
    lr.backward()
    tol = 1e-12 if precision == "fp64" else 2e-5
    assert abs(float(loss) - float(lr)) <= tol * float(lr)
    assert rel_rms(g.grad.cpu().numpy(), gr.grad.cpu().numpy()) < tol
    plan.close()


def test_finite_differences_image_and_gains():
    """Central differences (FP64, step 1e-3) of L = sum |g_i g_j* (A x) - V_obs|^2."""
    from rascil_gb300.autograd import apply_gains, predict
    c = _case("fp64", nants=16, ntimes=4, nchan=2, npix=64)
    plan = c["plan"]
    rng = numpy.random.default_rng(4)
    x0 = rng.normal(size=(1, 64, 64)) * 0.1
    g0 = (1 + 0.05 * rng.normal(size=(16, 2))) * numpy.exp(
        1j * rng.uniform(-numpy.pi / 8, numpy.pi / 8, (16, 2)))
    obs = torch.tensor(rng.normal(size=(plan.nrows, 2, 1)) + 1j * rng.normal(size=(plan.nrows, 2, 1)),
                       dtype=torch.complex128, device="cuda")

    def loss_of(x, g):
        v = apply_gains(predict(x, plan), g, c["a1"], c["a2"])
        return (v - obs).abs().pow(2).sum()

    x = torch.tensor(x0, device="cuda", requires_grad=True)
    g = torch.tensor(g0, dtype=torch.complex128, device="cuda", requires_grad=True)
    loss_of(x, g).backward()
    dx = rng.normal(size=x0.shape)
    dg = rng.normal(size=g0.shape) + 1j * rng.normal(size=g0.shape)
    h = 1e-3
    with torch.no_grad():
        xt, gt = torch.tensor(x0, device="cuda"), torch.tensor(g0, device="cuda")
        dxt, dgt = torch.tensor(dx, device="cuda"), torch.tensor(dg, device="cuda")
        fd_x = (loss_of(xt + h * dxt, gt) - loss_of(xt - h * dxt, gt)) / (2 * h)
        fd_g = (loss_of(xt, gt + h * dgt) - loss_of(xt, gt - h * dgt)) / (2 * h)
        h2 = h / 2
        fd_g2 = (loss_of(xt, gt + h2 * dgt) - loss_of(xt, gt - h2 * dgt)) / (2 * h2)
    an_x = float((x.grad * dxt).sum())
    an_g = float(torch.real((g.grad.conj() * dgt).sum()))
    # L is quadratic in x: central differences are exact up to rounding
    assert abs(float(fd_x) - an_x) <= 1e-8 * abs(an_x)
    # L is quartic in g: the O(h^2) truncation (~1e-5 relative at h = 1e-3) ...
    assert abs(float(fd_g) - an_g) <= 1e-4 * abs(an_g)
    # ... cancels in the Richardson combination of steps h and h/2
    rich = (4 * float(fd_g2) - float(fd_g)) / 3
    assert abs(rich - an_g) <= 1e-8 * abs(an_g)
    plan.close()


def test_gradient_descent_reduces_the_loss():
    """A few steps of gradient descent on the image recover a point source."""
    from rascil_gb300.autograd import predict
    c = _case("fp32", nants=24, ntimes=8, nchan=2, npix=64)
    plan = c["plan"]
    truth = torch.zeros((1, 64, 64), dtype=torch.float32, device="cuda")
    truth[0, 30, 37] = 1.0
    obs = predict(truth, plan).detach()
    x = torch.zeros_like(truth, requires_grad=True)
    losses = []
    for _ in range(8):
        x.grad = None
        loss = (predict(x, plan) - obs).abs().pow(2).sum()
        loss.backward()
        losses.append(float(loss))
        with torch.no_grad():  # steepest descent with exact line search on the quadratic
            g = x.grad
            ag = predict(g, plan)
            alpha = (g * g).sum() / (2 * ag.abs().pow(2).sum())
            x -= alpha * g
    assert losses[-1] < 0.1 * losses[0]
    assert int(torch.argmax(x.detach()).item()) == 30 * 64 + 37
    plan.close()


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp64", 1e-9)])
def test_predict_adjoint_dot_product_full_size(precision, tol):
    """The differentiable-predict configuration at its stated size: a 2048^2
    sky, 128 antennas (8,128 baselines) in a 1 km disk, 8 channels over
    150-158 MHz, 64 times (4,161,536 visibilities): Re<y, A x> = <x, A^H y>
    through the autograd Function (A^H = the gridder applied in backward)."""
    from rascil_gb300 import simulation as sim
    from rascil_gb300.autograd import predict
    from rascil_gb300.wgridder import Plan
    uvw, freq, pc, cfg = sim.observation("gain-solve", seed=0)
    assert uvw.shape[:2] == (64, 8128) and len(freq) == 8 and cfg["npixel"] == 2048
    fu = torch.from_numpy(uvw.reshape(-1, 3) * numpy.array([-1.0, 1.0, -1.0])).cuda()
    f = torch.from_numpy(freq.copy()).cuda()
    eps = 1e-5 if precision == "fp32" else 1e-12
    plan = Plan(fu, f, 2048, 2048, cfg["cellsize"], cfg["cellsize"], eps, True, npol=1,
                precision=precision)
    try:
        g = torch.Generator(device="cuda")
        g.manual_seed(3)
        x = torch.randn((1, 2048, 2048), generator=g, device="cuda",
                        dtype=plan.real_dtype).requires_grad_(True)
        y = torch.randn((plan.nrows, plan.nchan, 1, 2), generator=g, device="cuda",
                        dtype=plan.real_dtype)
        y = torch.view_as_complex(y).contiguous()
        v = predict(x, plan)
        lhs = torch.real(torch.vdot(y.reshape(-1).to(torch.complex128),
                                    v.reshape(-1).to(torch.complex128)))
        lhs.backward()
        rhs = (x.detach().double() * x.grad.double()).sum()
        # Cauchy-Schwarz scale of the inner product
        scale = float(torch.linalg.vector_norm(v.detach().to(torch.complex128)) *
                      torch.linalg.vector_norm(y.to(torch.complex128)))
        assert abs(float(lhs) - float(rhs)) <= tol * scale, (float(lhs), float(rhs), scale)
    finally:
        plan.close()
