"""The CPU-baseline leg of bench.py on CPU: the oversampling chooser and the
sampled invert + predict of the oracle's C gridder run on a small case, and
the chosen sample covers exactly the items whose support reaches a sampled
plane."""
import numpy
import pytest


def _case(n=20000, seed=0):
    rng = numpy.random.default_rng(seed)
    uvw = rng.uniform(-1, 1, (n, 3)) * numpy.array([3000.0, 3000.0, 400.0])
    freq = numpy.array([1.0e8, 1.2e8])
    s = freq / 299792458.0
    u = (uvw[:, 0:1] * s).ravel()
    v = (uvw[:, 1:2] * s).ravel()
    w = (uvw[:, 2:3] * s).ravel()
    return u, v, w


def test_sigma_chooser_returns_a_candidate_with_estimates():
    import bench
    u, v, w = _case()
    sigma, est = bench.cpu_choose_sigma(u, v, w, 128, 2e-3, 1e-5, 2)
    assert sigma in bench.CPU_SIGMAS and sigma in est
    assert all(t > 0 for t in est.values())
    assert est[sigma] == min(est.values())


def test_sampled_gridding_covers_the_items_reaching_the_planes():
    import bench
    from oracle import wgridder as owg
    u, v, w = _case(5000, seed=1)
    seen = {}

    def values(idx):
        seen["idx"] = idx
        return numpy.ones(idx.size, numpy.complex128)

    dt, plan, planes, n, est = bench.cpu_gridder_sample(u, v, w, values, numpy.zeros((64, 64)),
                                                        64, 4e-3, 1e-5, 3, 1.5, 2)
    assert dt > 0 and plan.sigma == 1.5 and len(planes) == 3 and n == seen["idx"].size
    assert est > dt  # the whole run holds more planes and item-planes than the sample
    ref = owg.Plan(64, 64, 4e-3, 4e-3, 1e-5, True, *owg.w_range(w, True), 1.5)
    a = numpy.ceil((numpy.abs(w) - ref.w_lo) / ref.dw)  # w < 0 items are mirrored
    reach = [i for i in range(w.size) if any(k - ref.W + 1 <= a[i] <= k for k in planes)]
    numpy.testing.assert_array_equal(seen["idx"], reach)


def test_unreachable_epsilon_is_an_error():
    import bench
    u, v, w = _case(2000)
    with pytest.raises(ValueError):
        bench.cpu_choose_sigma(u, v, w, 64, 4e-3, 1e-30, 1)
