#!/usr/bin/env python
"""Mvis/s of invert + predict (w-stacking gridder) on one GB300.

Workload (default): the LOW-like configuration -- 512 stations (224 uniform
in a 2 km disk, 288 log-radial 2-35 km; 130,816 baselines), 128 hour
angles over +-3 h, 16 channels over 100-200 MHz, 4 linear polarisations
(1,071,644,672 visibilities), complex64 data with float64 uvw, 1,000
point sources plus sigma=0.01 Jy noise, imaged MFS into an 8192^2
Stokes IQUV image (cell 1e-5 rad, epsilon 1e-5, w-stacking on).  All
data are seeded synthetic arrays of that shape.

A step is one pass of the hot path over the workload:
plan (w range, bucket sort) + invert (ms2dirty, 4 pols, linear -> IQUV)
+ predict (dirty2ms, IQUV -> linear), inputs resident in HBM.
Mvis/s = (vis inverted + vis predicted) / step time.

Reported alongside: the plain FP64 form on the same workload, relative
RMS errors of both forms against the FP64 direct DFT (at sampled rows and
pixels), the end-to-end rate through invert_ng / predict_ng with host
buffers, per-kernel device times with the HBM roofline of the dominant
kernel, the GPU clocks seen during the timed region and the CPU baseline
(the oracle's multithreaded C gridder on a bounded sample).

``--impl reference`` times the reference path's CPU stand-in alone.

``--path`` selects a path either side of the imaging step instead, each
with its own JSON line (device-timed rate, per-kernel GB/s, an end-to-end
rate through the public API with page-locked host arrays, and a timed CPU
oracle sample): ``weights`` (weight_visibility, uniform, over every sample
of the workload), ``rotation`` (gb_phase_rotate over the workload's
visibilities, and the imaging step with the rotation fused in against the
centred step), ``lists`` (invert_list / residual_list over 256 uneven
snapshots, at 1, 4 and 8 streams, with the device-busy time of one pass).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mvis/s invert+predict on 1 GB300, FP32 vs FP64 form at rel RMS<=1e-5 vs DFT"
SCALES = {
    # name: overrides of the configuration (None = as specified)
    "full": dict(ntimes=None, nchan=None, npixel=None),
    "medium": dict(ntimes=16, nchan=8, npixel=2048),
    "small": dict(ntimes=8, nchan=4, npixel=2048),
    "tiny": dict(ntimes=2, nchan=2, npixel=512),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb", choices=["gb", "reference"])
    ap.add_argument("--config", default="low-like")
    ap.add_argument("--scale", default="full", choices=list(SCALES))
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-planes", type=int, default=4,
                    help="w-planes in the CPU baseline sample")
    ap.add_argument("--grid-budget-gb", type=float, default=0.0,
                    help="memory for one batch of w-planes (0 = planner default)")
    ap.add_argument("--fp64-warmup", type=int, default=0,
                    help="untimed FP64-form steps (the FP32 warm-up already built the caches)")
    ap.add_argument("--tune", action="store_true",
                    help="run the per-shape autotuner first (untimed) and use its choice")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the per-shape autotuner (use cached or default plan parameters)")
    ap.add_argument("--plan", default=None,
                    help="fixed plan parameters sigma,tile,slab (e.g. 2,16,2); implies --no-tune")
    ap.add_argument("--fft-mode", default="auto", choices=["auto", "columns", "cufft2d"],
                    help="per-plane transforms of the FP32 form (auto: column kernels where "
                         "they apply)")
    ap.add_argument("--json-out", default=None)
    ap.add_argument("--path", default="imaging",
                    choices=["imaging", "weights", "rotation", "lists"],
                    help="imaging: the headline invert+predict step (default); weights: "
                         "imaging weights; rotation: the phase rotation (standalone kernel and "
                         "its cost fused into the imaging step); lists: the list workflows on "
                         "256 uneven snapshots")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        first = vis.split(",")[0].strip() if vis else ""
        self.index = int(first) if first.isdigit() else index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(numpy.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# workload

class Workload:
    def __init__(self, name, scale, device):
        import torch
        from rascil_gb300 import simulation as sim
        from rascil_gb300.polarisation import conversion_matrix, PolarisationFrame

        ov = SCALES[scale]
        uvw, freq, pc, cfg = sim.observation(name, seed=0, ntimes=ov["ntimes"],
                                             nchan=ov["nchan"], npixel=ov["npixel"])
        self.name, self.scale, self.cfg = name, scale, cfg
        self.uvw_host = uvw
        self.freq = freq
        self.phasecentre = pc
        self.ntimes, self.nbl, _ = uvw.shape
        self.nrows = self.ntimes * self.nbl
        self.nchan = len(freq)
        self.vis_pol = PolarisationFrame(cfg["pol"])
        self.img_pol = PolarisationFrame(cfg["image_pol"])
        self.npv = self.vis_pol.npol
        self.npol = self.img_pol.npol
        self.npixel = cfg["npixel"]
        self.cell = cfg["cellsize"]
        self.epsilon = cfg["epsilon"]
        self.nvis = self.nrows * self.nchan * self.npv
        self.pm_in = conversion_matrix(self.vis_pol, self.img_pol)
        self.pm_out = conversion_matrix(self.img_pol, self.vis_pol)
        self.src = sim.sources(cfg, seed=0)
        self.device = device
        # device copies: uvw as ng.py hands it to the gridder (u, w flipped)
        u = torch.from_numpy(uvw.reshape(-1, 3).copy()).to(device)
        self.uvw_raw = u.clone()
        u[:, 0].neg_()
        u[:, 2].neg_()
        self.uvw = u
        self.freq_dev = torch.from_numpy(freq.copy()).to(device)
        # model image (Stokes I of the sources at their pixels), [pol][y][x]
        model = numpy.zeros((self.npol, self.npixel, self.npixel), dtype=numpy.float32)
        ix, iy, l, m, flux = self.src
        numpy.add.at(model[0], (iy, ix), flux)
        self.model32 = torch.from_numpy(model).to(device)
        # visibilities of the sources (component DFT) plus noise, vis frame
        from rascil_gb300.dft import dft_components
        lmn = sim.lmn_rows(self.src)
        flux_v = sim.component_fluxes(cfg, self.src, self.nchan)
        vis = dft_components(self.uvw_raw, self.freq_dev, lmn, flux_v, precision="fp32",
                             exact=False)
        if cfg["noise"] > 0:
            g = torch.Generator(device=device)
            g.manual_seed(1234)
            noise = torch.randn(vis.shape + (2,), generator=g, device=device,
                                dtype=torch.float32) * cfg["noise"]
            vis += torch.view_as_complex(noise)
            del noise
        self.vis32 = vis.contiguous()
        self.wgt32 = torch.ones(vis.shape, dtype=torch.float32, device=device)
        self.lmn = lmn
        self.flux_v = flux_v
        torch.cuda.synchronize(device)


GRID_BUDGET = [0]
FFT_MODE = ["auto"]
FIXED_PLAN = [None]


def make_plan(wl, precision, params=None):
    from rascil_gb300.wgridder import Plan
    params = params or FIXED_PLAN[0] or {}
    return Plan(wl.uvw, wl.freq_dev, wl.npixel, wl.npixel, wl.cell, wl.cell, wl.epsilon, True,
                npol=wl.npol, precision=precision, grid_budget_bytes=GRID_BUDGET[0],
                sigma=params.get("sigma", 0.0), tile=params.get("tile", 0),
                slab=params.get("slab", 0), fft_mode=FFT_MODE[0])


def tune(wl, precision, vis, wgt, model):
    """Per-shape autotuning (untimed): the plan parameters the timed steps
    then pick up from the tuning cache."""
    from rascil_gb300 import tuning
    key = tuning.shape_key(wl.npixel, wl.npixel, wl.cell, wl.npol, precision, wl.epsilon, True,
                           wl.nrows, wl.nchan)
    best, timings = tuning.autotune(key, lambda prm: step(wl, precision, vis, wgt, model, prm))
    return {"key": key, "chosen": best, "candidate_ms": timings}


def step(wl, precision, vis, wgt, model, params=None):
    plan = make_plan(wl, precision, params)
    dirty = plan.ms2dirty(vis, wgt=wgt, polmat=wl.pm_in, layout="yx")
    pred = plan.dirty2ms(model, polmat=wl.pm_out, npol_vis=wl.npv, layout="yx")
    info = plan.info
    plan.close()
    return dirty, pred, info


def time_steps(wl, precision, vis, wgt, model, steps, warmup, sampler=None, profile=False):
    import torch
    from rascil_gb300 import _lib
    for _ in range(warmup):
        step(wl, precision, vis, wgt, model)
    torch.cuda.synchronize()
    if profile:
        _lib.profile_reset()
        _lib.profile_enable(True)
    if sampler:
        sampler.start()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record()
    out = None
    for _ in range(steps):
        out = step(wl, precision, vis, wgt, model)
    stop.record()
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    stats = None
    if profile:
        _lib.profile_enable(False)
        stats = _lib.profile_read()
    return start.elapsed_time(stop) / steps, out, clocks, stats


def accuracy(wl, dirty, pred, precision, nrows_check=512, npix_check=192):
    """Relative RMS vs the FP64 direct DFT: predict at sampled rows (all
    channels and pols), invert (Stokes I, unnormalised) at sampled pixels."""
    import torch
    from rascil_gb300.dft import dft_components, dft_pixels
    rng = numpy.random.default_rng(99)
    rows = numpy.sort(rng.choice(wl.nrows, size=min(nrows_check, wl.nrows), replace=False))
    rows_t = torch.from_numpy(rows).to(wl.device)
    truth = dft_components(wl.uvw_raw[rows_t].contiguous(), wl.freq_dev, wl.lmn, wl.flux_v,
                           precision="fp64", exact=True).cpu().numpy()
    got = pred[rows_t].to(torch.complex128).cpu().numpy()
    e_pred = float(numpy.linalg.norm(got - truth) / numpy.linalg.norm(truth))
    # invert: Stokes I visibilities (image frame) -> exact dirty values
    ix, iy = wl.src[0], wl.src[1]
    npx = wl.npixel
    rnd = rng.integers(0, npx, size=(npix_check, 2))
    pix = numpy.concatenate([numpy.stack([ix, iy], -1)[:npix_check], rnd])
    m = torch.from_numpy(wl.pm_in[0]).to(wl.device)  # row of the I pol
    vis = wl.vis32 if precision == "fp32" else wl.vis32.to(torch.complex128)
    visI = torch.einsum("q,rcq->rc", m.to(vis.dtype), vis).contiguous().unsqueeze(-1)
    truth_px = dft_pixels(wl.uvw, wl.freq_dev, visI.to(torch.complex128), None, pix, npx, npx,
                          wl.cell, wl.cell, True, exact=True).cpu().numpy()
    del visI
    d = dirty[0].double().cpu().numpy()
    got_px = d[pix[:, 1], pix[:, 0]]
    e_inv = float(numpy.linalg.norm(got_px - truth_px) / numpy.linalg.norm(truth_px))
    return {"predict_rel_rms": e_pred, "invert_rel_rms": e_inv,
            "sample": "predict: %d rows x %d chan x %d pol; invert: Stokes I at %d pixels "
                      "(%d source pixels + %d random)" % (len(rows), wl.nchan, wl.npv, len(pix),
                                                         min(npix_check, len(ix)), npix_check)}


def roofline(stats, peaks):
    mine = {k: v for k, v in stats.items() if not k.startswith("cufft")}
    total_ms = sum(v["ms"] for v in stats.values())
    dom = max(mine, key=lambda k: mine[k]["ms"])
    d = mine[dom]
    ach = d["bytes"] / (d["ms"] * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs")
    src = "of measured" if peak else "of fallback"
    peak = peak or 6800.0
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tpath):
        try:
            with open(tpath) as f:
                t = json.load(f)
            traffic = t.get(dom)
        except (OSError, ValueError):
            traffic = None
    kernels = {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                   "share": round(v["ms"] / total_ms, 4) if total_ms else None,
                   "gbs": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1) if v["ms"] else None}
               for k, v in sorted(stats.items(), key=lambda kv: -kv[1]["ms"])}
    return ({"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": peak,
             "unit": "GB/s", "frac": round(ach / peak, 4), "peak_source": src,
             "bytes_per_launch": d["bytes"] / d["launches"],
             "ms_per_launch": d["ms"] / d["launches"], "traffic": traffic}, kernels)


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's C gridder on a bounded sample

CPU_SIGMAS = (1.25, 1.5, 1.75, 2.0)
_CPU_SIGMA = {}  # workload -> (sigma, estimates): chosen once per process


def _sample_planes(nplanes, n):
    """n evenly spread interior planes: k_j = floor((j + 1/2) nplanes / n)."""
    return sorted(set(int((j + 0.5) * nplanes / n) for j in range(n)))


def _items_reaching(plan, w, planes):
    a = numpy.ceil((w - plan.w_lo) / plan.dw)
    keep = numpy.zeros(w.size, dtype=bool)
    for k in planes:
        keep |= (a >= k - plan.W + 1) & (a <= k)
    return numpy.nonzero(keep)[0]


def cpu_gridder_sample(u, v, w, values, model, npix, cell, eps, nplanes_sample, sigma, cores):
    """Invert + predict, on the CPU gridder, of the items whose support
    reaches an evenly spread subset of the w-planes: u, v, w in wavelengths
    (ng.py's sign flips applied), ``values(idx)`` gives those items' complex
    values, ``model`` is the [y][x] image.  Returns (seconds, plan, planes,
    items gridded)."""
    from oracle import cgridder
    from oracle import wgridder as owg
    plan = owg.Plan(npix, npix, cell, cell, eps, True, float(w.min()), float(w.max()), sigma)
    planes = _sample_planes(plan.nplanes, nplanes_sample)
    idx = _items_reaching(plan, w, planes)
    pr = cgridder.Prepared(plan, u[idx], v[idx], w[idx])
    vals = values(idx)
    t0 = time.perf_counter()
    cgridder.grid_items(pr, vals, cores, planes)
    cgridder.degrid_items(pr, model, cores, planes)
    return time.perf_counter() - t0, plan, planes, idx.size


def cpu_choose_sigma(u, v, w, npix, cell, eps, cores, nplanes_probe=2, sigmas=CPU_SIGMAS):
    """The grid oversampling the CPU gridder runs this workload fastest at,
    as ducc0 picks its kernel by a cost model (FFT volume grows about as
    sigma^3 with w-stacking, gridding work as W^3): per candidate, the
    sampled invert + predict of ``nplanes_probe`` planes with unit values,
    scaled by the candidate's plane count.  Returns (sigma, {sigma: s})."""
    est = {}
    model = numpy.zeros((npix, npix))
    for sg in sigmas:
        try:
            dt, plan, planes, _ = cpu_gridder_sample(
                u, v, w, lambda idx: numpy.ones(idx.size, numpy.complex128), model, npix, cell,
                eps, nplanes_probe, sg, cores)
        except (ValueError, IndexError):
            continue  # no kernel reaches eps at this sigma
        est[sg] = dt * plan.nplanes / len(planes)
    if not est:
        raise ValueError("no CPU gridder oversampling reaches epsilon %g" % eps)
    return min(est, key=est.get), est


def cpu_sample(wl, nplanes_sample):
    """Invert + predict of the full workload restricted to an evenly spread
    subset of w-planes, one polarisation, FP64 on all host cores, at the
    oversampling fastest on the CPU; returns (extrapolated Mvis/s, cores,
    description, measured seconds)."""
    import torch
    from oracle import cgridder
    s = wl.freq / 299792458.0
    uvw = wl.uvw.cpu().numpy()  # flipped, as ng.py passes to ducc0
    u = (uvw[:, 0:1] * s).ravel()
    v = (uvw[:, 1:2] * s).ravel()
    w = (uvw[:, 2:3] * s).ravel()
    cores = cgridder.max_threads()
    key = (wl.name, wl.scale)
    if key not in _CPU_SIGMA:
        try:
            _CPU_SIGMA[key] = cpu_choose_sigma(u, v, w, wl.npixel, wl.cell, wl.epsilon, cores)
        except Exception as e:  # the choice is an optimisation: keep the measured default
            print("cpu_choose_sigma failed (%s); the CPU baseline uses sigma 2" % e,
                  file=sys.stderr)
            _CPU_SIGMA[key] = (2.0, {})
    sigma, est = _CPU_SIGMA[key]
    m = torch.from_numpy(wl.pm_in[0]).to(wl.device)

    def values(idx):  # Stokes I of the chosen items, formed on the device
        vi = wl.vis32.to(torch.complex128) @ m
        return vi.reshape(-1)[torch.from_numpy(idx).to(wl.device)].cpu().numpy()

    model = wl.model32[0].double().cpu().numpy()
    dt, plan, planes, nitems = cpu_gridder_sample(u, v, w, values, model, wl.npixel, wl.cell,
                                                  wl.epsilon, nplanes_sample, sigma, cores)
    # scale: all planes, all polarisations (ng.py grids each pol separately)
    t_full = dt * plan.nplanes / len(planes) * wl.npol
    mvis = 2 * wl.nvis / t_full / 1e6
    why = ("the fastest on these cores of %s, estimated s per pol: %s"
           % ("/".join("%g" % x for x in CPU_SIGMAS),
              ", ".join("%g: %.0f" % kv for kv in sorted(est.items())))
           if est else "the oversampling choice failed; the default")
    desc = ("oracle C gridder (FP64, OpenMP + scipy.fft pocketfft) at sigma %g, W %d (%s), "
            "invert+predict of Stokes I over %d of %d w-planes (%d items reach them), time "
            "scaled by %d/%d planes x %d pols: %.1f s measured"
            % (sigma, plan.W, why, len(planes), plan.nplanes, nitems, plan.nplanes, len(planes),
               wl.npol, dt))
    return mvis, cores, desc, dt


# ---------------------------------------------------------------------------

def e2e_run(wl, steps):
    """invert_ng + predict_ng on a host-resident BlockVisibility / Image."""
    import torch
    from rascil_gb300 import simulation as sim
    from rascil_gb300.imaging import invert_ng, predict_ng
    from rascil_gb300.imaging.ng import clear_plan_cache
    from rascil_gb300.data_models import BlockVisibility
    from rascil_gb300.polarisation import PolarisationFrame

    def pinned(shape, dtype):  # numpy view of page-locked host memory
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    shape = (wl.ntimes, wl.nbl, wl.nchan, wl.npv)
    vis_host = pinned(shape, torch.complex64)
    torch.from_numpy(vis_host).copy_(wl.vis32.reshape(shape))
    flags = pinned(shape, torch.int64)
    flags[...] = 0
    wgt = pinned(shape, torch.float64)
    wgt[...] = 1.0
    uvw = pinned(wl.uvw_host.shape, torch.float64)
    uvw[...] = wl.uvw_host
    # natural weighting: imaging weights are the weights (one shared array)
    bvis = BlockVisibility(vis_host, uvw, wl.freq, wl.phasecentre,
                           PolarisationFrame(wl.cfg["pol"]), flags=flags, weight=wgt,
                           imaging_weight=wgt)
    model = sim.model_image(wl.cfg, wl.src, wl.phasecentre, wl.freq)
    kw = dict(epsilon=wl.epsilon, precision="fp32", do_wstacking=True)

    def one():
        # one plan per step, as in the device-timed steps: invert builds it,
        # predict reuses it through the API's plan cache
        clear_plan_cache()
        im, sw = invert_ng(bvis, model, **kw)
        pv = predict_ng(bvis, model, **kw)
        return im, pv

    one()  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    h2d = (vis_host.nbytes + flags.nbytes + wgt.nbytes + 2 * uvw.nbytes
           + model["pixels"].data.nbytes)
    d2h = vis_host.nbytes + model["pixels"].data.nbytes
    return {"value": round(2 * wl.nvis / dt / 1e6, 3), "unit": "Mvis/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "s_per_step": round(dt, 3), "steps": steps,
            "api": "rascil_gb300.imaging.invert_ng + predict_ng (precision='fp32') on a "
                   "host BlockVisibility (page-locked arrays) / Image"}


# ---------------------------------------------------------------------------
# the paths either side of the imaging step (--path): each prints its own line

def _ptr(t):
    import ctypes
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _event_loop(fn, steps, warmup, sampler=None, profile=True):
    """ms per call of fn() timed with CUDA events on the current stream
    (after warm-up), with the per-kernel profile of the timed calls."""
    import torch
    from rascil_gb300 import _lib
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    if profile:
        _lib.profile_reset()
        _lib.profile_enable(True)
    if sampler:
        sampler.start()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    stats = None
    if profile:
        _lib.profile_enable(False)
        stats = _lib.profile_read()
    return a.elapsed_time(b) / steps, clocks, stats


def _aux_line(args, metric, value, unit, ms, workload, roof, kernels, clocks, launches, **extra):
    line = {"path": args.path, "metric": metric, "value": round(value, 3), "unit": unit,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (seeded)", "config": workload, "clocks": clocks,
            "roofline": roof, "gpu_launches": launches, "kernels": kernels}
    line.update(extra)
    return line


def bench_weights(args):
    """weight_visibility (uniform, the reference's default) over every
    sample of the workload: gb_weight_visibility on device-resident arrays,
    then end to end on a host BlockVisibility."""
    import torch
    from rascil_gb300 import _lib
    from rascil_gb300 import simulation as sim
    from rascil_gb300.data_models import BlockVisibility
    from rascil_gb300.imaging import weight_visibility
    from rascil_gb300.polarisation import PolarisationFrame
    device = torch.device("cuda", torch.cuda.current_device())
    lib = _lib.load()
    ov = SCALES[args.scale]
    uvw, freq, pc, cfg = sim.observation(args.config, seed=0, ntimes=ov["ntimes"],
                                         nchan=ov["nchan"], npixel=ov["npixel"])
    nt, nbl, _ = uvw.shape
    R, C, P = nt * nbl, len(freq), PolarisationFrame(cfg["pol"]).npol
    npix, cell = cfg["npixel"], cfg["cellsize"]
    nvis = R * C * P
    g = torch.Generator(device=device)
    g.manual_seed(7)
    uvw_d = torch.from_numpy(uvw.reshape(-1, 3).copy()).to(device)
    freq_d = torch.from_numpy(freq.copy()).to(device)
    weight = torch.rand((R, C, P), generator=g, device=device, dtype=torch.float64).add_(0.5)
    imw = torch.rand((R, C, P), generator=g, device=device, dtype=torch.float64)
    imw.mul_(0.4).add_(0.8).mul_(weight)
    flags = (torch.rand((R, C, P), generator=g, device=device) < 0.05).to(torch.int64)
    v2i = torch.zeros(C, dtype=torch.int32, device=device)  # MFS image: one channel
    grid = torch.empty((1, npix, npix, P), dtype=torch.float64, device=device)
    cells = torch.empty((R, C), dtype=torch.int32, device=device)
    out = torch.empty_like(weight)
    sums = torch.empty(2, dtype=torch.float64, device=device)
    cdx, cdy = -numpy.degrees(cell), numpy.degrees(cell)
    stream = torch.cuda.current_stream(device)

    def call(scheme, robustness=0.0):
        _lib.check(lib.gb_weight_visibility(
            _ptr(uvw_d), _ptr(freq_d), R, C, P, _ptr(v2i), 1, npix, npix, cdx, cdy, _ptr(weight),
            _ptr(imw), _ptr(flags), _lib.GB_FLAGS_I64, scheme, robustness, _ptr(grid),
            _ptr(cells), _ptr(out), _ptr(sums), _ptr_stream(stream)), "gb_weight_visibility")

    sampler = ClockSampler(device.index)
    ms, clocks, stats = _event_loop(lambda: call(_lib.GB_WEIGHT_UNIFORM), args.steps,
                                    args.warmup, sampler)
    roof, kernels = roofline(stats, load_peaks())
    launches = sum(v["launches"] for v in stats.values()) // args.steps
    others = {}
    for name, scheme, rob in (("natural", _lib.GB_WEIGHT_NATURAL, 0.0),
                              ("robust_0", _lib.GB_WEIGHT_ROBUST, 0.0)):
        m, _, _ = _event_loop(lambda: call(scheme, rob), args.steps, 1, profile=False)
        others[name] = {"ms": round(m, 3), "value": round(nvis / (m * 1e-3) / 1e6, 1)}
    # CPU baseline: the oracle (numpy, the reference's own algorithm) on the
    # first 1/64 of the rows
    from oracle import weighting as ow
    rs = max(1, R // 64)
    sl = slice(0, rs)
    hw = weight[sl].cpu().numpy()
    him = imw[sl].cpu().numpy()
    hf = flags[sl].cpu().numpy()
    t0 = time.perf_counter()
    ow.weight_visibility(uvw.reshape(-1, 3)[sl], freq, hw, him, hf, numpy.zeros(C, int), 1, npix,
                         npix, cdx, cdy, "uniform")
    cpu_dt = time.perf_counter() - t0
    cpu = {"value": round(rs * C * P / cpu_dt / 1e6, 3), "unit": "Mvis/s", "cores": 1,
           "kind": "port", "sample": "oracle/weighting.py (numpy, uniform) on the first %d of %d "
           "rows (%d samples): %.1f s" % (rs, R, rs * C * P, cpu_dt)}
    del hw, him, hf
    # end to end: weight_visibility on a host BlockVisibility (page-locked arrays)
    def pinned_from(t):
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t)
        return h.numpy()

    shape = (nt, nbl, C, P)
    bvis = BlockVisibility(torch.empty(shape, dtype=torch.complex64, pin_memory=True).numpy(),
                           pinned_from(uvw_d).reshape(nt, nbl, 3), freq, pc,
                           PolarisationFrame(cfg["pol"]),
                           flags=pinned_from(flags).reshape(shape),
                           weight=pinned_from(weight).reshape(shape),
                           imaging_weight=pinned_from(imw).reshape(shape))
    model = sim.model_image(cfg, ([], [], [], [], []), pc, freq)
    del weight, imw, flags, out, grid, cells
    torch.cuda.empty_cache()
    weight_visibility(bvis, model, weighting="uniform")  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        weight_visibility(bvis, model, weighting="uniform")
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / args.e2e_steps
    e2e = {"value": round(nvis / dt / 1e6, 3), "unit": "Mvis/s",
           "h2d_bytes_per_step": int(3 * 8 * nvis + 24 * R),
           "d2h_bytes_per_step": int(8 * nvis), "s_per_step": round(dt, 3),
           "api": "rascil_gb300.imaging.weight_visibility(bvis, model, 'uniform') on page-locked "
                  "host arrays (weight, imaging_weight, int64 flags, uvw)"}
    workload = {"workload": "imaging weights (uniform) of %s %s: %d rows x %d chan x %d pol "
                            "onto the %d^2 MFS uv grid (cell %g rad)"
                            % (args.config, args.scale, R, C, P, npix, cell),
                "nvis": nvis, "l2": "inputs larger than L2 (%.1f GB f64 weights and flags)"
                                    % (3 * 8 * nvis / 1e9)}
    return _aux_line(args, "Mvis/s imaging weights (weight_visibility, uniform) on 1 GB300",
                     nvis / (ms * 1e-3) / 1e6, "Mvis/s", ms, workload, roof, kernels, clocks,
                     launches, dtype="f64", schemes=others, cpu_baseline=cpu, e2e=e2e)


def bench_rotation(args):
    """The phase rotation: gb_phase_rotate over the workload's complex64
    visibilities in place, and the imaging step with an image centred 0.01
    rad away from the phase centre (rotation fused into the plan) against
    the centred step."""
    import torch
    from rascil_gb300 import _lib
    from rascil_gb300.data_models import BlockVisibility, SkyDirection
    from rascil_gb300.imaging.base import phaserotate_visibility, phasor_direction
    from rascil_gb300.polarisation import PolarisationFrame
    from rascil_gb300.wgridder import Plan
    device = torch.device("cuda", torch.cuda.current_device())
    lib = _lib.load()
    wl = Workload(args.config, args.scale, device)
    new = SkyDirection(wl.phasecentre.ra.rad + 0.01, wl.phasecentre.dec.rad - 0.005)
    s = phasor_direction(new, wl.phasecentre)
    stream = torch.cuda.current_stream(device)
    vis = wl.vis32.clone()
    flip = [0]

    def call():
        flip[0] ^= 1  # forward, then inverse: the data stay bounded
        _lib.check(lib.gb_phase_rotate(_ptr(wl.uvw_raw), _ptr(wl.freq_dev), wl.nrows, wl.nchan,
                                       wl.npv, _ptr(vis), _lib.GB_FP32, s[0], s[1], s[2], flip[0],
                                       _ptr_stream(stream)), "gb_phase_rotate")

    sampler = ClockSampler(device.index)
    ms, clocks, stats = _event_loop(call, args.steps, args.warmup, sampler)
    roof, kernels = roofline(stats, load_peaks())
    del vis
    torch.cuda.empty_cache()

    # fused: the imaging step with and without the shift (plan-frame coefficients)
    def imaging_step(shift):
        plan = Plan(wl.uvw, wl.freq_dev, wl.npixel, wl.npixel, wl.cell, wl.cell, wl.epsilon,
                    True, npol=wl.npol, precision="fp32", phase_shift=shift)
        plan.ms2dirty(wl.vis32, wgt=wl.wgt32, polmat=wl.pm_in, layout="yx")
        plan.dirty2ms(wl.model32, polmat=wl.pm_out, npol_vis=wl.npv, layout="yx")
        plan.close()

    fused = {}
    for name, shift in (("centred", (0.0, 0.0, 0.0)), ("offset", (-s[0], s[1], -s[2]))):
        m, _, _ = _event_loop(lambda: imaging_step(shift), 2, 1, profile=False)
        fused[name + "_ms"] = round(m, 1)
    fused["note"] = ("plan + invert + predict of the whole workload; 'offset' images 0.01 rad "
                     "from the phase centre with the rotation fused into the item factors")
    # CPU baseline: the oracle rotation (numpy) on the first 1/64 of the rows
    from oracle import rotation as orot
    rs = max(1, wl.nrows // 64)
    hv = wl.vis32[:rs].cpu().numpy()
    t0 = time.perf_counter()
    orot.phaserotate(hv, wl.uvw_host.reshape(-1, 3)[:rs], wl.freq, (s[0], s[1], s[2]))
    cpu_dt = time.perf_counter() - t0
    cpu = {"value": round(rs * wl.nchan * wl.npv / cpu_dt / 1e6, 3), "unit": "Mvis/s",
           "cores": 1, "kind": "port",
           "sample": "oracle/rotation.py (numpy) on the first %d of %d rows: %.1f s"
                     % (rs, wl.nrows, cpu_dt)}
    # end to end: phaserotate_visibility on a host BlockVisibility (page-locked vis)
    shape = (wl.ntimes, wl.nbl, wl.nchan, wl.npv)
    hvis = torch.empty(shape, dtype=torch.complex64, pin_memory=True)
    hvis.copy_(wl.vis32.reshape(shape))
    bvis = BlockVisibility(hvis.numpy(), wl.uvw_host, wl.freq, wl.phasecentre,
                           PolarisationFrame(wl.cfg["pol"]))
    phaserotate_visibility(bvis, new)  # warm-up
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        phaserotate_visibility(bvis, new)
    dt = (time.perf_counter() - t0) / args.e2e_steps
    e2e = {"value": round(wl.nvis / dt / 1e6, 3), "unit": "Mvis/s",
           "h2d_bytes_per_step": int(8 * wl.nvis + 24 * wl.nrows),
           "d2h_bytes_per_step": int(8 * wl.nvis), "s_per_step": round(dt, 3),
           "api": "rascil_gb300.imaging.base.phaserotate_visibility on a host BlockVisibility "
                  "(includes the reference's deep copy of the other arrays)"}
    workload = dict(workload_config(wl))
    workload["workload"] = "phase rotation of " + workload["workload"]
    return _aux_line(args, "Mvis/s phase rotation (gb_phase_rotate, complex64 in place) on 1 "
                     "GB300", wl.nvis / (ms * 1e-3) / 1e6, "Mvis/s", ms, workload, roof, kernels,
                     clocks, 1, dtype="f32", fused_in_imaging=fused, cpu_baseline=cpu, e2e=e2e)


def bench_lists(args):
    """invert_list / residual_list over 256 uneven snapshots (the batched configuration:
    32-512 antennas, 1-8 channels, 1-16 times, 256-2048 pixel images),
    page-locked host BlockVisibility per snapshot, FP32 form at eps 1e-5.
    Timed with the host clock: every call ends with its results on the host."""
    import torch
    from rascil_gb300 import simulation as sim
    from rascil_gb300.data_models import BlockVisibility, SkyDirection, create_image
    from rascil_gb300.imaging.ng import clear_plan_cache
    from rascil_gb300.polarisation import PolarisationFrame
    from rascil_gb300 import workflows as wf
    snaps = sim.snapshot_batch(256)
    rng = numpy.random.default_rng(3)
    pc = SkyDirection(0.0, numpy.radians(-45.0))
    blocks, models = [], []
    for sn in snaps:
        nt, nbl, _ = sn["uvw"].shape
        shape = (nt, nbl, len(sn["freq"]), 1)
        vis = torch.empty(shape, dtype=torch.complex64, pin_memory=True).numpy()
        vis[...] = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(numpy.complex64)
        blocks.append(BlockVisibility(vis, sn["uvw"], sn["freq"], pc, PolarisationFrame("stokesI")))
        bw = sn["freq"].max() - sn["freq"].min() + 1.0
        models.append(create_image(sn["npix"], sn["cell"], pc, frequency=[sn["freq"].mean()],
                                   channel_bandwidth=[bw]))
    nvis = sum(sn["nvis"] for sn in snaps)
    kw = dict(epsilon=1e-5, precision="fp32")

    def timed(fn):
        clear_plan_cache(release_memory=True)
        torch.cuda.empty_cache()
        fn()  # warm-up
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return float(numpy.median(ts))

    res = {}
    for streams in (1, 4, 8):
        dt = timed(lambda: wf.invert_list_rsexecute_workflow(blocks, models, "ng",
                                                             streams=streams, **kw))
        res["invert_list_streams_%d" % streams] = {"s": round(dt, 3),
                                                   "value": round(nvis / dt / 1e6, 2)}
    dt_res = timed(lambda: wf.residual_list_rsexecute_workflow(blocks, models, "ng", streams=4,
                                                               **kw))

    def composed():
        mv = wf.predict_list_rsexecute_workflow(wf.zero_list_rsexecute_workflow(blocks), models,
                                                "ng", streams=4, **kw)
        return wf.invert_list_rsexecute_workflow(wf.subtract_list_rsexecute_workflow(blocks, mv),
                                                 models, "ng", streams=4, **kw)

    dt_comp = timed(composed)
    res["residual_list_fused_streams_4"] = {"s": round(dt_res, 3),
                                            "value": round(2 * nvis / dt_res / 1e6, 2)}
    res["residual_list_composed_streams_4"] = {"s": round(dt_comp, 3),
                                               "value": round(2 * nvis / dt_comp / 1e6, 2)}
    # device time of one sequential pass, per kernel: how much of the list's
    # wall time the GPU is busy
    from rascil_gb300 import _lib
    clear_plan_cache(release_memory=True)
    _lib.profile_reset()
    _lib.profile_enable(True)
    t0 = time.perf_counter()
    wf.invert_list_rsexecute_workflow(blocks, models, "ng", streams=1, **kw)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    _lib.profile_enable(False)
    stats = _lib.profile_read()
    busy = sum(v["ms"] for v in stats.values()) / 1e3
    top = sorted(stats.items(), key=lambda kv: -kv[1]["ms"])[:6]
    res["device_profile_streams_1"] = {
        "wall_s": round(wall, 3), "kernel_s": round(busy, 3),
        "top": {k: {"ms": round(v["ms"], 1), "launches": v["launches"]} for k, v in top}}
    clear_plan_cache(release_memory=True)
    best = max((v["value"], k) for k, v in res.items() if k.startswith("invert_list"))
    # CPU baseline: the oracle's C gridder (ms2dirty, FP64, all cores) over
    # the first snapshots until ~10 s of work
    from oracle import cgridder
    done, t_cpu = 0, 0.0
    for sn, b in zip(snaps, blocks):
        if t_cpu > 10.0:
            break
        u = sn["uvw"].reshape(-1, 3).copy()
        u[:, 0] *= -1.0
        u[:, 2] *= -1.0
        ms_ = b["vis"].data.reshape(u.shape[0], -1).astype(numpy.complex128)
        t0 = time.perf_counter()
        cgridder.ms2dirty(u, sn["freq"], ms_, None, sn["npix"], sn["npix"], sn["cell"],
                          sn["cell"], 1e-5, True)
        t_cpu += time.perf_counter() - t0
        done += sn["nvis"]
    cpu = {"value": round(done / t_cpu / 1e6, 3), "unit": "Mvis/s",
           "cores": cgridder.max_threads(), "kind": "port",
           "sample": "oracle C gridder ms2dirty (FP64, OpenMP) on the first %d vis of the list: "
                     "%.1f s" % (done, t_cpu)}
    workload = {"workload": "invert_list over 256 snapshots (32-512 antennas in 1 km, 1-8 chan "
                            "in 100-200 MHz, 1-16 times, 256-2048 px, cell 1/(2.2 max|uv|)), "
                            "eps 1e-5, FP32 form, Stokes I, page-locked host arrays",
                "nvis": int(nvis), "snapshots": len(snaps)}
    t_best = res[best[1]]["s"]
    return _aux_line(args, "Mvis/s invert_list over 256 uneven snapshots on 1 GB300 (host data)",
                     best[0], "Mvis/s", t_best * 1e3, workload, None, None, None, None,
                     dtype="f32", best=best[1], runs=res, cpu_baseline=cpu,
                     e2e={"value": best[0], "unit": "Mvis/s",
                          "h2d_bytes_per_step": int(8 * nvis + 24 * sum(
                              sn["uvw"].shape[0] * sn["uvw"].shape[1] for sn in snaps)),
                          "d2h_bytes_per_step": int(sum(8 * sn["npix"] ** 2 for sn in snaps))},
                     timing="host clock around each whole list call (results on the host)")


def _ptr_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


AUX_PATHS = {"weights": bench_weights, "rotation": bench_rotation, "lists": bench_lists}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def dist_setup(args):
    if args.gpus <= 1 or "RANK" not in os.environ:
        return 0, 1
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    world = int(os.environ["WORLD_SIZE"])
    if torch.cuda.is_available():
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world


def max_over_ranks(x, world):
    """The slowest rank's value (every rank gets it): the job's step time is
    the max over ranks.  NCCL reduces a CUDA tensor, gloo a CPU one."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    """CPU stand-in for the reference path (ducc0 is not installable here)."""
    rank, world = dist_setup(args)
    if rank != 0:
        return None
    import torch
    device = torch.device("cuda", 0) if torch.cuda.is_available() else None
    if device is None:
        print(json.dumps({"impl": "reference", "unavailable": "workload generation needs a GPU"}))
        return None
    wl = Workload(args.config, args.scale, device)
    times = []
    res = None
    for i in range(args.warmup + args.steps):
        res = cpu_sample(wl, args.cpu_planes)
        if i >= args.warmup:
            times.append(2 * wl.nvis / (res[0] * 1e6))
    mvis, cores, desc, _ = res
    t = float(numpy.mean(times))
    value = 2 * wl.nvis / t / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mvis/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t * 1e3, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": workload_config(wl),
            "cpu_baseline": {"value": round(value, 4), "unit": "Mvis/s", "cores": cores,
                             "kind": "port", "sample": desc},
            "e2e": {"value": round(value, 4), "unit": "Mvis/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "ducc0 0.24.0 (the reference's gridder) is not installed on this image; "
                    "the timed stand-in is the oracle's C restatement of the same algorithm"}
    print(json.dumps(line))
    return line


def workload_config(wl):
    cfg = wl.cfg
    nants = int(round((1 + numpy.sqrt(1 + 8 * wl.nbl)) / 2))
    return {"workload": "%s %s: %d stations, %d baselines x %d times, %d chan %.0f-%.0f MHz, "
                        "%s -> %s, %d^2 image, cell %g rad, eps %g, w-stacking"
                        % (wl.name, wl.scale, nants, wl.nbl, wl.ntimes, wl.nchan,
                           wl.freq[0] / 1e6, wl.freq[-1] / 1e6, cfg["pol"], cfg["image_pol"],
                           wl.npixel, wl.cell, wl.epsilon),
            "nvis": wl.nvis, "nrows": wl.nrows, "nchan": wl.nchan, "npol": wl.npv,
            "npixel": wl.npixel, "epsilon": wl.epsilon,
            "l2": "inputs larger than L2 (vis %.1f GB per step)" % (wl.nvis * 8 / 1e9)}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.path != "imaging":
        line = AUX_PATHS[args.path](args)
        print(json.dumps(line))
        if args.json_out:
            with open(args.json_out, "w") as f:
                json.dump(line, f, indent=1)
        return
    import torch
    GRID_BUDGET[0] = int(args.grid_budget_gb * (1 << 30))
    FFT_MODE[0] = args.fft_mode
    if args.plan:
        sg, tl, sb = args.plan.split(",")
        FIXED_PLAN[0] = {"sigma": float(sg), "tile": int(tl), "slab": int(sb)}
        args.no_tune = True
    rank, world = dist_setup(args)
    device = torch.device("cuda", torch.cuda.current_device())
    from rascil_gb300 import _lib
    _lib.load()
    wl = Workload(args.config, args.scale, device)
    sampler = ClockSampler(device.index) if rank == 0 else None
    tuned = tune(wl, "fp32", wl.vis32, wl.wgt32, wl.model32) if args.tune and not args.no_tune \
        else None
    if world > 1:
        torch.distributed.barrier()
    ms, out, clocks, stats = time_steps(wl, "fp32", wl.vis32, wl.wgt32, wl.model32, args.steps,
                                        args.warmup, sampler=sampler, profile=True)
    ms = max_over_ranks(ms, world)
    dirty, pred, info = out
    value = world * 2 * wl.nvis / (ms * 1e-3) / 1e6
    acc32 = accuracy(wl, dirty, pred, "fp32")
    del dirty, pred, out
    roof, kernels = roofline(stats, load_peaks())
    launches = sum(v["launches"] for k, v in stats.items() if not k.startswith("cufft"))
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mvis/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded arrays, 1000 point sources via GPU DFT + noise)",
            "config": workload_config(wl), "clocks": clocks, "roofline": roof,
            "gpu_launches": int(launches / args.steps),
            "accuracy_fp32": acc32,
            "plan": {k: info[k] for k in ("support", "sigma", "ngrid_x", "nplanes",
                                          "planes_per_batch", "tile", "slab", "beta", "dw",
                                          "fft_mode")},
            "tuning": tuned,
            "kernels": kernels}
    torch.cuda.empty_cache()
    if not args.no_fp64:
        vis64 = wl.vis32.to(torch.complex128)
        wgt64 = wl.wgt32.double()
        model64 = wl.model32.double()
        ms64, out64, _, _ = time_steps(wl, "fp64", vis64, wgt64, model64, args.fp64_steps,
                                       args.fp64_warmup)
        acc64 = accuracy(wl, out64[0], out64[1], "fp64")
        line["fp64_form"] = {"value": round(world * 2 * wl.nvis / (ms64 * 1e-3) / 1e6, 3),
                             "unit": "Mvis/s", "ms_per_step": round(ms64, 2),
                             "steps": args.fp64_steps, "accuracy": acc64,
                             "fp32_over_fp64": round(ms64 / ms, 3)}
        del vis64, wgt64, model64, out64
        torch.cuda.empty_cache()
    if not args.no_e2e and rank == 0:
        line["e2e"] = e2e_run(wl, args.e2e_steps)
        torch.cuda.empty_cache()
    if not args.no_cpu and rank == 0:
        try:
            mvis, cores, desc, dt = cpu_sample(wl, args.cpu_planes)
            line["cpu_baseline"] = {"value": round(mvis, 4), "unit": "Mvis/s", "cores": cores,
                                    "kind": "port", "sample": desc}
        except Exception as e:  # reported in the line, not fatal to the GPU measurement
            line["cpu_baseline"] = {"value": None, "unit": "Mvis/s", "cores": None,
                                    "kind": "port", "sample": "failed: %s" % e}
    if rank == 0:
        print(json.dumps(line))
        if args.json_out:
            with open(args.json_out, "w") as f:
                json.dump(line, f, indent=1)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
