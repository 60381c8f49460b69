"""The allocation-free w-range entry point, through the C-ABI.

gb_wrange_noalloc serves callers that cannot allocate device memory where
they need the w range (a host framework that owns every device buffer, a
real-time pipeline that forbids allocation after start-up): its scratch is
a fixed device array inside the library.  It must give the same w range
as the planner's own reduction (gb_plan_create, read back through
gb_plan_info_get), bit for bit, on consecutive calls with different data
(the shared scratch keeps the previous call's contents).

This file is named to be collected last.
"""
import ctypes

import numpy
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _problem(seed, nrows, nchan):
    rng = numpy.random.default_rng(seed)
    uvw = rng.uniform(-1, 1, (nrows, 3)) * numpy.array([5000.0, 5000.0, 3000.0 * (seed + 1)])
    freq = numpy.linspace(0.9e8, 1.9e8 + 1e7 * seed, nchan)
    return (torch.from_numpy(uvw).to("cuda"), torch.from_numpy(freq).to("cuda"))


def test_wrange_noalloc_matches_planner_twice():
    from rascil_gb300 import _lib, wgridder
    lib = _lib.load()
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    # the wider w range over many rows first (49 partials), then fewer rows
    # (3 partials) whose w range lies strictly inside it: a reduction that
    # read the first call's leftover partials would widen the second range
    raw = []
    for seed, nrows, nchan in ((1, 200_003, 7), (0, 9_000, 3)):
        uvw, freq = _problem(seed, nrows, nchan)
        raw.append((float(uvw[:, 2].min()), float(uvw[:, 2].max())))
        if len(raw) == 2:  # the case is meaningful only if the second range is inside
            assert raw[0][0] < raw[1][0] and raw[1][1] < raw[0][1]
        plan = wgridder.Plan(uvw, freq, 64, 64, 2e-3, 2e-3, 1e-5, True, precision="fp32")
        ref = plan.info
        plan.close()
        stream = wgridder._stream(uvw.device)
        _lib.check(lib.gb_wrange_noalloc(ctypes.c_void_p(uvw.data_ptr()),
                                         ctypes.c_void_p(freq.data_ptr()), nrows, nchan,
                                         ctypes.c_void_p(out.data_ptr()), stream),
                   "gb_wrange_noalloc")
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert got[0] == ref["w_lo"] and got[1] == ref["w_hi"], (got, ref["w_lo"], ref["w_hi"])
        assert got[2] == 0.0 and got[3] == 0.0


def test_wrange_noalloc_rejects_oversize_input():
    from rascil_gb300 import _lib
    lib = _lib.load()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    rc = lib.gb_wrange_noalloc(p, p, 67_108_864 + 1, 1, p, None)
    assert rc == _lib.GB_ERR_INVALID_ARG
    assert b"exceed" in lib.gb_last_error_string()
