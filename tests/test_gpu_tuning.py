"""The per-shape autotuner on the GPU: its bounded search from the
planner's choice over grid oversampling, tile, slab and planes per batch,
the cached winner reused by every later plan of that shape, and a recorded
choice changing the plan (ducc0 picks its kernel internally per call, as
rascil/processing_components/imaging/ng.py:91-103,232-248 call it; here the
choice is measured and cached)."""
import numpy
import pytest

from oracle import dft as odft
from tests.cases import random_problem, rel_rms

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture
def tuning(tmp_path, monkeypatch):
    from rascil_gb300 import tuning as t
    monkeypatch.setenv("RASCIL_GB300_TUNING", str(tmp_path / "tuning.json"))
    monkeypatch.setattr(t, "_mem", {})
    monkeypatch.setattr(t, "_loaded", [False])
    return t


def _problem():
    c = random_problem(seed=4, nrow=4000, nchan=2, npix=128, pixsize=2e-3, wscale=600.0)
    u = torch.from_numpy(c["uvw"]).cuda()
    f = torch.from_numpy(c["freq"]).cuda()
    vis = torch.from_numpy(c["ms"]).to(device="cuda", dtype=torch.complex64)
    img = torch.from_numpy(c["img"][:1]).to(device="cuda", dtype=torch.float32)
    return c, u, f, vis, img


def _plan(c, u, f, **kw):
    from rascil_gb300.wgridder import Plan
    return Plan(u, f, c["npix"], c["npix"], c["pixsize"], c["pixsize"], 1e-5, True,
                precision="fp32", **kw)


def test_autotune_searches_caches_and_changes_the_plan(tuning):
    c, u, f, vis, img = _problem()
    key = tuning.shape_key(c["npix"], c["npix"], c["pixsize"], 1, "fp32", 1e-5, True,
                           u.shape[0], f.shape[0])

    def run(prm):
        p = _plan(c, u, f, sigma=prm["sigma"], tile=prm["tile"], slab=prm["slab"],
                  planes_per_batch=prm["planes"])
        p.ms2dirty(vis, layout="xy")
        p.dirty2ms(img, layout="xy")
        p.close()

    p0 = _plan(c, u, f, bind=False)
    info = p0.info
    p0.close()
    start = {"sigma": info["sigma"], "tile": info["tile"], "slab": info["slab"],
             "planes": info["planes_per_batch"]}
    best, timings = tuning.autotune(key, run, start=start, max_seconds=60.0)
    timed = [k for k, v in timings.items() if v is not None]
    assert len(timed) >= 6, timings
    # the search varied more than sigma
    varied = {k.split(",")[i].split("=")[0] for k in timed for i in range(4)
              if k.split(",")[i] != timed[0].split(",")[i]}
    assert {"sigma", "tile", "slab"} <= varied, timings
    assert min(v for v in timings.values() if v is not None) == timings[tuning._name(best)]
    # the cached winner is what a plan of this shape now uses
    chosen = tuning.choose(key, c["npix"], c["npix"], u.shape[0], f.shape[0])
    assert chosen["sigma"] == best["sigma"] and chosen["tile"] == best["tile"]
    p = _plan(c, u, f)
    assert (p.info["sigma"], p.info["tile"], p.info["slab"]) == (best["sigma"], best["tile"],
                                                               best["slab"])
    p.close()
    # a recorded choice changes the plan, and the results stay exact
    tuning.autotune(key, run, candidates=[{"sigma": 1.5, "tile": 16, "slab": 2, "planes": 3}])
    p = _plan(c, u, f)
    assert (p.info["sigma"], p.info["tile"], p.info["slab"],
            p.info["planes_per_batch"]) == (1.5, 16, 2, 3)
    got = p.ms2dirty(vis, layout="xy")[0].double().cpu().numpy()
    p.close()
    ref = odft.ms2dirty_dft(c["uvw"], c["freq"], c["ms"][..., 0], None, c["npix"], c["npix"],
                            c["pixsize"], c["pixsize"], True)
    assert rel_rms(got, ref) < 1e-5
    # the choice persists for a fresh process state
    tuning._mem.clear()
    tuning._loaded[0] = False
    assert tuning.choose(key, c["npix"], c["npix"], u.shape[0], f.shape[0]) == {
        "sigma": 1.5, "tile": 16, "slab": 2, "planes": 3}
