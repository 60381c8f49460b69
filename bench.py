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
    ap.add_argument("--config", default="c2")
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

def cpu_sample(wl, nplanes_sample):
    """Invert + predict of the full workload restricted to an evenly spread
    subset of w-planes, one polarisation, FP64 on all host cores; returns
    (extrapolated Mvis/s, cores, description)."""
    import torch
    from oracle import cgridder
    from oracle import wgridder as owg
    s = wl.freq / 299792458.0
    uvw = wl.uvw.cpu().numpy()  # flipped, as ng.py passes to ducc0
    u = (uvw[:, 0:1] * s).ravel()
    v = (uvw[:, 1:2] * s).ravel()
    w = (uvw[:, 2:3] * s).ravel()
    plan = owg.Plan(wl.npixel, wl.npixel, wl.cell, wl.cell, wl.epsilon, True, float(w.min()),
                    float(w.max()))
    nplanes = plan.nplanes
    # evenly spread interior planes: k_j = floor((j + 1/2) nplanes / n)
    planes = sorted(set(int((j + 0.5) * nplanes / nplanes_sample) for j in range(nplanes_sample)))
    # keep only items whose support reaches a sampled plane
    a = numpy.ceil((w - plan.w_lo) / plan.dw)
    keep = numpy.zeros(w.size, dtype=bool)
    for k in planes:
        keep |= (a >= k - plan.W + 1) & (a <= k)
    idx = numpy.nonzero(keep)[0]
    pr = cgridder.Prepared(plan, u[idx], v[idx], w[idx])
    vis_i = (wl.vis32.to(torch.complex128) @ torch.from_numpy(wl.pm_in[0]).to(wl.device)
             ).reshape(-1)[torch.from_numpy(idx).to(wl.device)].cpu().numpy()
    model = wl.model32[0].double().cpu().numpy()
    cores = cgridder.max_threads()
    t0 = time.perf_counter()
    cgridder.grid_items(pr, vis_i, cores, planes)
    cgridder.degrid_items(pr, model, cores, planes)
    dt = time.perf_counter() - t0
    # scale: all planes, all polarisations (ng.py grids each pol separately)
    t_full = dt * nplanes / len(planes) * wl.npol
    mvis = 2 * wl.nvis / t_full / 1e6
    desc = ("oracle C gridder (FP64, OpenMP + scipy.fft pocketfft), invert+predict of Stokes I "
            "over %d of %d w-planes (%d items reach them), time scaled by %d/%d planes x %d "
            "pols: %.1f s measured" % (len(planes), nplanes, idx.size, nplanes, len(planes),
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
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world


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
    if world > 1:
        t = torch.tensor([ms], device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
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
        mvis, cores, desc, dt = cpu_sample(wl, args.cpu_planes)
        line["cpu_baseline"] = {"value": round(mvis, 4), "unit": "Mvis/s", "cores": cores,
                                "kind": "port", "sample": desc}
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
