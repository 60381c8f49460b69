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
    # the medium visibilities at twice the image side: about the full
    # workload's items per (w-slab, uv-tile) bucket (buckets grow as the
    # fourth power of the image side, tiles and w-planes each as its square)
    "medium-wide": dict(ntimes=16, nchan=8, npixel=4096),
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
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-planes", type=int, default=4,
                    help="w-planes in the CPU baseline sample")
    ap.add_argument("--ref-planes", type=int, default=2,
                    help="w-planes in each step's sample of --impl reference (about 4-8 s a "
                         "step on 16 cores, so 25 steps end within a few minutes)")
    ap.add_argument("--grid-budget-gb", type=float, default=0.0,
                    help="memory for one batch of w-planes (0 = planner default)")
    ap.add_argument("--fp64-warmup", type=int, default=0,
                    help="untimed FP64-form steps (the FP32 warm-up already built the caches)")
    ap.add_argument("--tune", action="store_true",
                    help="run the per-shape autotuner first (untimed) and use its choice")
    ap.add_argument("--tune-seconds", type=float, default=120.0,
                    help="time budget of the autotuner's search")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the per-shape autotuner (use cached or default plan parameters)")
    ap.add_argument("--plan", default=None,
                    help="fixed plan parameters sigma,tile,slab (e.g. 2,16,2); implies --no-tune")
    ap.add_argument("--fft-mode", default="auto", choices=["auto", "columns", "cufft2d"],
                    help="per-plane transforms of the FP32 form (auto: column kernels where "
                         "they apply)")
    ap.add_argument("--no-mid", action="store_true",
                    help="skip the MID-like configuration's rate and accuracy")
    ap.add_argument("--mid-steps", type=int, default=2)
    ap.add_argument("--mid-warmup", type=int, default=1)
    ap.add_argument("--no-reduced", action="store_true",
                    help="skip the reduced-case accuracy of every form (GPU and CPU)")
    ap.add_argument("--json-out", default=None)
    ap.add_argument("--path", default="imaging",
                    choices=["imaging", "weights", "rotation", "lists", "batch", "autograd",
                             "dft"],
                    help="imaging: the headline invert+predict step (default); weights: "
                         "imaging weights; rotation: the phase rotation (standalone kernel and "
                         "its cost fused into the imaging step); lists: the list workflows on "
                         "256 uneven snapshots; batch: the 256 uneven snapshots as one batched "
                         "device program; autograd: 200 gradient-descent steps of the "
                         "differentiable predict; dft: the component DFT against the "
                         "reference's own CUDA kernel")
    ap.add_argument("--gd-steps", type=int, default=200)
    ap.add_argument("--nsnap", type=int, default=256)
    ap.add_argument("--nslots", type=int, default=8)
    ap.add_argument("--e2e-gd-steps", type=int, default=20)
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

class CpuWorkload:
    """The workload's geometry, sources and model image on the host (numpy
    only): everything the CPU legs need, built without the GPU library."""

    def __init__(self, name, scale):
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
        # model image (Stokes I of the sources at their pixels), [pol][y][x]
        model = numpy.zeros((self.npol, self.npixel, self.npixel), dtype=numpy.float32)
        ix, iy, l, m, flux = self.src
        numpy.add.at(model[0], (iy, ix), flux)
        self.model_host = model

    def flipped_uvw(self):
        """uvw [nrows, 3] as ng.py hands them to the gridder (u, w negated)."""
        u = self.uvw_host.reshape(-1, 3).copy()
        u[:, 0] *= -1.0
        u[:, 2] *= -1.0
        return u


class Workload:
    """The workload on the device: uvw, frequencies, the model image and the
    sources' visibilities (GPU component DFT) plus noise."""

    def __init__(self, name, scale, device, cpu=None):
        import torch
        cw = cpu or CpuWorkload(name, scale)
        for k in ("name", "scale", "cfg", "uvw_host", "freq", "phasecentre", "ntimes", "nbl",
                  "nrows", "nchan", "vis_pol", "img_pol", "npv", "npol", "npixel", "cell",
                  "epsilon", "nvis", "pm_in", "pm_out", "src"):
            setattr(self, k, getattr(cw, k))
        cfg = self.cfg
        from rascil_gb300 import simulation as sim
        self.device = device
        # device copies: uvw as ng.py hands it to the gridder (u, w flipped)
        u = torch.from_numpy(self.uvw_host.reshape(-1, 3).copy()).to(device)
        self.uvw_raw = u.clone()
        u[:, 0].neg_()
        u[:, 2].neg_()
        self.uvw = u
        self.freq_dev = torch.from_numpy(self.freq.copy()).to(device)
        self.model32 = torch.from_numpy(cw.model_host).to(device)
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


def make_plan(wl, precision, params=None, bind=True):
    from rascil_gb300.wgridder import Plan
    params = params or FIXED_PLAN[0] or {}
    return Plan(wl.uvw, wl.freq_dev, wl.npixel, wl.npixel, wl.cell, wl.cell, wl.epsilon, True,
                npol=wl.npol, precision=precision, grid_budget_bytes=GRID_BUDGET[0],
                sigma=params.get("sigma", 0.0), tile=params.get("tile", 0),
                slab=params.get("slab", 0), planes_per_batch=params.get("planes", 0),
                fft_mode=FFT_MODE[0], bind=bind)


def tune(wl, precision, vis, wgt, model, max_seconds=120.0):
    """Per-shape autotuning (untimed): a coordinate search from the
    planner's own choice over sigma, tile, slab and planes per batch; the
    timed steps then pick the winner up from the tuning cache."""
    from rascil_gb300 import tuning
    key = tuning.shape_key(wl.npixel, wl.npixel, wl.cell, wl.npol, precision, wl.epsilon, True,
                           wl.nrows, wl.nchan)
    tuning.forget(key)
    p0 = make_plan(wl, precision, bind=False)
    info = p0.info
    p0.close()
    start = {"sigma": info["sigma"], "tile": info["tile"], "slab": info["slab"],
             "planes": info["planes_per_batch"]}
    plane_bytes = info["ngrid_x"] * info["ngrid_y"] * wl.npol * (8 if precision == "fp32"
                                                                  else 16)
    best, timings = tuning.autotune(key, lambda prm: step(wl, precision, vis, wgt, model, prm),
                                    start=start, plane_bytes=plane_bytes,
                                    max_seconds=max_seconds)
    return {"key": key, "planner_choice": start, "chosen": best, "candidate_ms": timings}


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


def _ncu_traffic(kernel):
    """profiles/ncu_traffic.json: per kernel, the DRAM bytes ncu measured per
    launch over the algorithmic bytes this bench counts for the same launches
    (captured on a smaller case of the same kernel)."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError, AttributeError):
        return None


# update-rate rooflines: shared-memory instructions per (item, pol, cell) update
UPDATE_COST = {"k_grid": ("atomics", 2.0, "2 conflict-free 32-bit shared atomic adds (re, im)"),
               "k_degrid": ("loads", 1.0, "1 8-byte grid read (complex64) through the L1 data "
                                         "pipe, against that pipe's conflict-free 8-byte "
                                         "shared-load rate")}


def roofline(stats, peaks, smem=None):
    mine = {k: v for k, v in stats.items() if not k.startswith("cufft")}
    total_ms = sum(v["ms"] for v in stats.values())
    dom = max(mine, key=lambda k: mine[k]["ms"])
    d = mine[dom]
    ach = d["bytes"] / (d["ms"] * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs")
    src = "of measured" if peak else "of fallback"
    peak = peak or 6800.0
    bpl = d["bytes"] / d["launches"]
    t = _ncu_traffic(dom)
    traffic = None
    if t and t.get("dram_over_algorithmic"):
        traffic = round(t["dram_over_algorithmic"] * bpl, 1)
    kernels = {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                   "share": round(v["ms"] / total_ms, 4) if total_ms else None,
                   "bytes": v["bytes"],
                   "gbs": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1) if v["ms"] else None}
               for k, v in sorted(stats.items(), key=lambda kv: -kv[1]["ms"])}
    secondary = {}
    for k, (what, per, desc) in UPDATE_COST.items():
        v = stats.get(k)
        if not v or not v.get("updates") or not v["ms"]:
            continue
        ups = v["updates"] / (v["ms"] * 1e-3)
        kernels[k]["updates_per_s"] = ups
        entry = {"updates_per_s": ups, "cost": desc}
        if smem:
            pk = (smem[0] if what == "atomics" else smem[1]) / per
            entry.update({"peak_updates_per_s": pk, "frac": round(ups / pk, 4),
                          "peak_source": "measured shared-memory %s rate of this GPU "
                                         "(gb_probe_smem_peaks)" % what})
        secondary[k] = entry
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": peak,
            "unit": "GB/s", "frac": round(ach / peak, 4), "peak_source": src,
            "bytes_per_launch": bpl, "ms_per_launch": d["ms"] / d["launches"],
            "traffic": traffic,
            "traffic_basis": (None if traffic is None else
                              "ncu dram__bytes_read+write / algorithmic bytes = %.3f on %s, "
                              "times this launch's algorithmic bytes"
                              % (t["dram_over_algorithmic"], t.get("case", "?"))),
            "secondary": secondary}
    return roof, kernels


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's C gridder on a bounded sample

CPU_SIGMAS = (1.25, 1.5, 1.75, 2.0)
_CPU_SIGMA = {}  # workload -> (sigma, estimates): chosen once per process
_CPU_COORDS = {}  # (config, scale): item u, v, w in wavelengths
_CPU_PREP = {}  # (config, scale, planes, sigma): a prepared sample and the model


def _sample_planes(nplanes, n):
    """n evenly spread interior planes: k_j = floor((j + 1/2) nplanes / n)."""
    return sorted(set(int((j + 0.5) * nplanes / n) for j in range(n)))


def _items_reaching(plan, w, planes):
    a = numpy.ceil((numpy.abs(w) - plan.w_lo) / plan.dw)  # w-stacking mirrors w < 0
    keep = numpy.zeros(w.size, dtype=bool)
    for k in planes:
        keep |= (a >= k - plan.W + 1) & (a <= k)
    return numpy.nonzero(keep)[0]


def cpu_gridder_prepare(u, v, w, values, npix, cell, eps, nplanes_sample, sigma):
    """The untimed part of a CPU sample: the plan, an evenly spread subset of
    its w-planes, the items whose support reaches them, their prepared
    coordinates and their values (``values(idx)``).  u, v, w in wavelengths
    (ng.py's sign flips applied)."""
    from oracle import cgridder
    from oracle import wgridder as owg
    plan = owg.Plan(npix, npix, cell, cell, eps, True, *owg.w_range(w, True), sigma)
    planes = _sample_planes(plan.nplanes, nplanes_sample)
    idx = _items_reaching(plan, w, planes)
    pr = cgridder.Prepared(plan, u[idx], v[idx], w[idx])
    return {"plan": plan, "planes": planes, "nreach": idx.size, "pr": pr,
            "vals": values(idx), "nitems": w.size}


def cpu_gridder_run(prep, model, cores):
    """Invert + predict, on the CPU gridder, of a prepared sample (``model``
    is the [y][x] image).  Returns (seconds, plan, planes, items gridded,
    estimated seconds of the whole invert + predict).

    The estimate scales the two parts of the measured time separately: the
    per-plane transforms and screens by (all planes / sampled planes), the
    spreading and gathering by (all item-planes / sampled item-planes),
    every item reaching W planes -- the sampled planes may hold more or
    fewer items than the average plane."""
    from oracle import cgridder
    plan, planes = prep["plan"], prep["planes"]
    timing = {}
    t0 = time.perf_counter()
    cgridder.grid_items(prep["pr"], prep["vals"], cores, planes, timing)
    cgridder.degrid_items(prep["pr"], model, cores, planes, timing)
    dt = time.perf_counter() - t0
    est = dt * plan.nplanes / len(planes)  # fallback: plane scaling alone
    if timing.get("item_planes"):
        est = (timing.get("planes", 0.0) * plan.nplanes / len(planes)
               + timing["items"] * (2.0 * prep["nitems"] * plan.W) / timing["item_planes"]
               + (dt - timing.get("planes", 0.0) - timing["items"]))
    return dt, plan, planes, prep["nreach"], est


def cpu_gridder_sample(u, v, w, values, model, npix, cell, eps, nplanes_sample, sigma, cores):
    """Prepare and run one CPU sample (see cpu_gridder_prepare / _run)."""
    prep = cpu_gridder_prepare(u, v, w, values, npix, cell, eps, nplanes_sample, sigma)
    return cpu_gridder_run(prep, model, cores)


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
            _, plan, planes, _, full = cpu_gridder_sample(
                u, v, w, lambda idx: numpy.ones(idx.size, numpy.complex128), model, npix, cell,
                eps, nplanes_probe, sg, cores)
        except (ValueError, IndexError):
            continue  # no kernel reaches eps at this sigma
        est[sg] = full
    if not est:
        raise ValueError("no CPU gridder oversampling reaches epsilon %g" % eps)
    return min(est, key=est.get), est


def cpu_sample(cw, nplanes_sample, nplanes_probe=2):
    """Invert + predict of the full workload restricted to an evenly spread
    subset of w-planes, one polarisation, FP64 on all host cores, at the
    oversampling fastest on the CPU.  Host only (``cw`` is a CpuWorkload):
    the sampled items' values are seeded complex Gaussians (the gridder's
    time does not depend on them).  Returns a dict: the extrapolated Mvis/s,
    cores, description, measured seconds, the full-step estimate and the
    oversampling used."""
    from oracle import cgridder
    key = (cw.name, cw.scale)
    if key not in _CPU_COORDS:  # host preparation, untimed, once per workload
        s = cw.freq / 299792458.0
        uvw = cw.flipped_uvw()  # as ng.py passes to ducc0
        _CPU_COORDS[key] = ((uvw[:, 0:1] * s).ravel(), (uvw[:, 1:2] * s).ravel(),
                            (uvw[:, 2:3] * s).ravel())
    u, v, w = _CPU_COORDS[key]
    cores = cgridder.max_threads()
    if key not in _CPU_SIGMA:
        try:
            _CPU_SIGMA[key] = cpu_choose_sigma(u, v, w, cw.npixel, cw.cell, cw.epsilon, cores,
                                               nplanes_probe)
        except (ValueError, IndexError, OSError) as e:  # an optimisation: keep the default
            print("cpu_choose_sigma failed (%s); the CPU baseline uses sigma 2" % e,
                  file=sys.stderr)
            _CPU_SIGMA[key] = (2.0, {})
    sigma, est = _CPU_SIGMA[key]

    def values(idx):
        rng = numpy.random.default_rng(11)
        return rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)

    pkey = key + (nplanes_sample, sigma)
    if pkey not in _CPU_PREP:  # untimed, once per sample shape; steps reuse it
        _CPU_PREP[pkey] = (cpu_gridder_prepare(u, v, w, values, cw.npixel, cw.cell,
                                               cw.epsilon, nplanes_sample, sigma),
                           cw.model_host[0].astype(numpy.float64))
    prep, model = _CPU_PREP[pkey]
    dt, plan, planes, nitems, t_pol = cpu_gridder_run(prep, model, cores)
    # scale: all planes and item-planes, all polarisations (ng.py grids each
    # pol separately)
    scale = t_pol / dt * cw.npol
    t_full = dt * scale
    mvis = 2 * cw.nvis / t_full / 1e6
    why = ("the fastest on these cores of %s, estimated s per pol: %s"
           % ("/".join("%g" % x for x in CPU_SIGMAS),
              ", ".join("%g: %.0f" % kv for kv in sorted(est.items())))
           if est else "the oversampling choice failed; the default")
    desc = ("oracle C gridder (FP64, OpenMP + scipy.fft pocketfft) at sigma %g, W %d (%s), "
            "invert+predict of one polarisation over %d of %d w-planes (%d items reach them; "
            "seeded Gaussian values), %.2f s measured; the transforms scaled by %d/%d planes, "
            "the spreading and gathering by all item-planes over the sampled ones, x %d pols"
            % (sigma, plan.W, why, len(planes), plan.nplanes, nitems, dt, plan.nplanes,
               len(planes), cw.npol))
    return {"mvis": mvis, "cores": cores, "desc": desc, "sample_s": dt, "full_s": t_full,
            "scale": scale, "sigma": sigma, "W": plan.W, "planes": len(planes),
            "nplanes": plan.nplanes}


# The reduced case on which both arms state their error against the exact
# DFT at the same epsilon: the workload's geometry (every baseline, its
# frequency band), 2 times x 4 channels, a 1024^2 image at the configured
# cell, Stokes I of its first 64 sources.
REDUCED = dict(ntimes=2, nchan=4, npixel=1024, nsrc=64, npix_check=128, nrows_check=256)


def reduced_case(name):
    """Host arrays of the reduced accuracy case: flipped uvw, freq, Stokes I
    visibilities [nrows, nchan] (exact FP64 component DFT, the oracle), the
    model image [y][x], the sampled pixels and rows with their exact
    invert / predict values (oracle direct sums)."""
    from oracle import dft as odft
    from rascil_gb300 import simulation as sim
    uvw, freq, pc, cfg = sim.observation(name, seed=0, ntimes=REDUCED["ntimes"],
                                         nchan=REDUCED["nchan"], npixel=REDUCED["npixel"])
    cfg = dict(cfg, nsrc=REDUCED["nsrc"])
    ix, iy, l, m, flux = sim.sources(cfg, seed=0)
    n = numpy.sqrt(1.0 - l * l - m * m)
    lmn = numpy.stack([l, m, n - 1.0], -1)
    uvw_lambda = uvw[:, :, None, :] * (freq / odft.SPEED_OF_LIGHT)[None, None, :, None]
    vis = odft.dft_cpu_looped(lmn, uvw_lambda, (flux / n)[:, None, None] *
                              numpy.ones((1, len(freq), 1)))[..., 0]
    vis = vis.reshape(-1, len(freq))
    npix, cell = cfg["npixel"], cfg["cellsize"]
    model = numpy.zeros((npix, npix))
    numpy.add.at(model, (iy, ix), flux)
    fu = uvw.reshape(-1, 3) * numpy.array([-1.0, 1.0, -1.0])
    rng = numpy.random.default_rng(5)
    k = REDUCED["npix_check"] // 2
    pix = numpy.concatenate([numpy.stack([ix, iy], -1)[:k], rng.integers(0, npix, (k, 2))])
    truth_px = odft.ms2dirty_dft(fu, freq, vis, None, npix, npix, cell, cell, True,
                                 pixel_subset=(pix[:, 0], pix[:, 1]), chunk=16)
    rows = numpy.sort(rng.choice(fu.shape[0], REDUCED["nrows_check"], replace=False))
    truth_v = odft.dirty2ms_dft(fu, freq, model.T, None, cell, cell, True, row_subset=rows)
    return dict(uvw=fu, freq=freq, vis=vis, model=model, npix=npix, cell=cell,
                eps=cfg["epsilon"], pix=pix, truth_px=truth_px, rows=rows, truth_v=truth_v,
                desc="%s geometry, %d times x %d baselines x %d chan, %d^2 image (cell %g), "
                     "Stokes I of %d sources; invert at %d pixels, predict at %d rows x %d "
                     "chan, against the oracle's FP64 direct sums"
                     % (name, uvw.shape[0], uvw.shape[1], len(freq), npix, cell, len(flux),
                        len(pix), len(rows), len(freq)))


def _rel(a, b):
    a, b = numpy.asarray(a), numpy.asarray(b)
    return float(numpy.linalg.norm((a - b).ravel()) / numpy.linalg.norm(b.ravel()))


def cpu_accuracy(rc, sigma, cores):
    """The CPU path's own error on the reduced case at the same epsilon: the
    oracle's C gridder (FP64, every w-plane) at the CPU's oversampling."""
    from oracle import cgridder
    dirty = cgridder.ms2dirty(rc["uvw"], rc["freq"], rc["vis"], None, rc["npix"], rc["npix"],
                              rc["cell"], rc["cell"], rc["eps"], True, nthreads=cores,
                              sigma=sigma)
    got_px = dirty[rc["pix"][:, 0], rc["pix"][:, 1]]
    pred = cgridder.dirty2ms(rc["uvw"][rc["rows"]], rc["freq"], rc["model"].T, None, rc["cell"],
                             rc["cell"], rc["eps"], True, nthreads=cores, sigma=sigma)
    return {"invert_rel_rms": _rel(got_px, rc["truth_px"]),
            "predict_rel_rms": _rel(pred, rc["truth_v"]),
            "form": "oracle C gridder FP64, sigma %g" % sigma}


def gpu_accuracy(rc, precision, device):
    """The GPU forms' error on the reduced case (Plan: invert + predict)."""
    import torch
    from rascil_gb300.wgridder import Plan
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    rdt = torch.float64 if precision == "fp64" else torch.float32
    u = torch.from_numpy(rc["uvw"]).to(device)
    f = torch.from_numpy(rc["freq"].copy()).to(device)
    plan = Plan(u, f, rc["npix"], rc["npix"], rc["cell"], rc["cell"], rc["eps"], True, npol=1,
                precision=precision)
    try:
        vis = torch.from_numpy(rc["vis"]).to(device=device, dtype=cdt).reshape(plan.nrows,
                                                                             plan.nchan, 1)
        dirty = plan.ms2dirty(vis, layout="xy")[0].double().cpu().numpy()
        model = torch.from_numpy(rc["model"].T.copy()).to(device=device, dtype=rdt)
        pred = plan.dirty2ms(model.reshape(1, rc["npix"], rc["npix"]), layout="xy")
        pred = pred[torch.from_numpy(rc["rows"]).to(device), :, 0].to(torch.complex128)
        info = plan.info
    finally:
        plan.close()
    return {"invert_rel_rms": _rel(dirty[rc["pix"][:, 0], rc["pix"][:, 1]], rc["truth_px"]),
            "predict_rel_rms": _rel(pred.cpu().numpy(), rc["truth_v"]),
            "form": "%s, sigma %g, W %d" % (precision, info["sigma"], info["support"])}


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

    split = {"invert_ng": 0.0, "predict_ng": 0.0}

    def one():
        # one plan per step, as in the device-timed steps: invert builds it,
        # predict reuses it through the API's plan cache; each call returns
        # host arrays, so it has finished on the device when it returns
        clear_plan_cache()
        t = time.perf_counter()
        im, sw = invert_ng(bvis, model, **kw)
        t1 = time.perf_counter()
        pv = predict_ng(bvis, model, **kw)
        split["invert_ng"] += t1 - t
        split["predict_ng"] += time.perf_counter() - t1
        return im, pv

    one()  # warm-up
    split.update(invert_ng=0.0, predict_ng=0.0)
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
            "s_per_call": {k: round(v / steps, 3) for k, v in split.items()},
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
        # the list as one device program on `streams` workspace slots
        dt = timed(lambda: wf.invert_list_rsexecute_workflow(blocks, models, "ng",
                                                             streams=streams, **kw))
        res["invert_list_streams_%d" % streams] = {"s": round(dt, 3),
                                                   "value": round(nvis / dt / 1e6, 2)}
    dt = timed(lambda: wf.invert_list_rsexecute_workflow(blocks, models, "ng", streams=4,
                                                         program=False, **kw))
    res["invert_list_thread_map_streams_4"] = {"s": round(dt, 3),
                                               "value": round(nvis / dt / 1e6, 2)}
    dt = timed(lambda: wf.predict_list_rsexecute_workflow(blocks, models, "ng", streams=8, **kw))
    res["predict_list_streams_8"] = {"s": round(dt, 3), "value": round(nvis / dt / 1e6, 2)}
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
    best = max((v["value"], k) for k, v in res.items() if k.startswith("invert_list_streams"))
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


def _blob_sky(npix, cell, nsrc, nblob, seed):
    """The differentiable-predict sky: ``nsrc`` point sources U[0.01, 1] Jy at
    pixel centres plus ``nblob`` circular Gaussian blobs (sigma 3-10 px,
    peak U[0.01, 1] Jy, cut at 4 sigma), [y][x] float64, within the inner
    half of the image."""
    rng = numpy.random.default_rng(seed)
    sky = numpy.zeros((npix, npix))
    lo, hi = npix // 4, 3 * npix // 4
    ix = rng.integers(lo, hi, nsrc)
    iy = rng.integers(lo, hi, nsrc)
    numpy.add.at(sky, (iy, ix), rng.uniform(0.01, 1.0, nsrc))
    for _ in range(nblob):
        sg = rng.uniform(3.0, 10.0)
        cx, cy = rng.integers(lo, hi, 2)
        r = int(4 * sg)
        yy, xx = numpy.mgrid[cy - r:cy + r + 1, cx - r:cx + r + 1]
        amp = rng.uniform(0.01, 1.0)
        sky[cy - r:cy + r + 1, cx - r:cx + r + 1] += amp * numpy.exp(
            -((xx - cx) ** 2 + (yy - cy) ** 2) / (2 * sg * sg))
    return sky


def bench_autograd(args):
    """The differentiable predict at its stated size: a 2048^2 FP32 sky
    (200 points + 20 Gaussian blobs), 128 antennas in a 1 km disk, 8
    channels over 150-158 MHz, 64 times, Stokes I, per-antenna per-channel
    gains (amplitude 1 + N(0, 0.05), phase U(-pi/8, pi/8)) applied as
    g_i conj(g_j); loss sum |V_pred - V_obs|^2 with V_obs from the FP64
    DFT of the sky under the true gains.  Timed: 200 gradient-descent steps
    on the image and the gains (forward dirty2ms + gains, backward = the
    gridder + the gain-gradient kernel), one plan for the run."""
    import torch
    from rascil_gb300 import _lib
    from rascil_gb300 import simulation as sim
    from rascil_gb300.autograd import apply_gains, baseline_antennas, predict
    from rascil_gb300.dft import dft_components
    from rascil_gb300.wgridder import Plan
    device = torch.device("cuda", torch.cuda.current_device())
    _lib.load()
    uvw, freq, pc, cfg = sim.observation("gain-solve", seed=0)
    nt, nbl, _ = uvw.shape
    nants = int(round((1 + numpy.sqrt(1 + 8 * nbl)) / 2))
    npix, cell, eps = cfg["npixel"], cfg["cellsize"], cfg["epsilon"]
    R, C = nt * nbl, len(freq)
    nvis = R * C
    sky = _blob_sky(npix, cell, 200, 20, seed=4)
    raw = torch.from_numpy(uvw.reshape(-1, 3).copy()).to(device)
    fu = raw.clone()
    fu[:, 0].neg_()
    fu[:, 2].neg_()
    f = torch.from_numpy(freq.copy()).to(device)
    # V_obs: FP64 DFT over every nonzero sky pixel (flux / n at its l, m),
    # the exact image-plane operator, then the true gains
    iy, ix = numpy.nonzero(sky)
    l = -(ix - npix // 2) * cell
    m = (iy - npix // 2) * cell
    n = numpy.sqrt(1.0 - l * l - m * m)
    lmn = numpy.stack([l, m, n - 1.0], -1)
    flux = (sky[iy, ix] / n)[:, None, None] * numpy.ones((1, C, 1))
    t0 = time.perf_counter()
    v_true = dft_components(raw, f, lmn, flux, precision="fp64", exact=True)
    torch.cuda.synchronize()
    t_dft = time.perf_counter() - t0
    rng = numpy.random.default_rng(9)
    g_true = (1 + 0.05 * rng.normal(size=(nants, C))) * numpy.exp(
        1j * rng.uniform(-numpy.pi / 8, numpy.pi / 8, (nants, C)))
    a1, a2 = baseline_antennas(nants, nt, device)
    gt = torch.from_numpy(g_true).to(device)
    obs = apply_gains(v_true, gt, a1, a2).to(torch.complex64).contiguous()
    del v_true
    plan = Plan(fu, f, npix, npix, cell, cell, eps, True, npol=1, precision="fp32")
    # image step 1 / L: L = 2 lambda_max(A^H A) (power iteration through the
    # plan's own predict and adjoint) with a margin for gains near 1
    with torch.no_grad():
        xp = torch.randn((1, npix, npix), device=device, dtype=torch.float32)
        lam = 1.0
        for _ in range(12):
            xp = plan.ms2dirty(plan.dirty2ms(xp, layout="yx"), layout="yx")
            lam = float(torch.linalg.vector_norm(xp))
            xp /= lam
    lr_x = 1.0 / (2.0 * lam * 1.25)
    a1l, a2l = a1.long(), a2.long()

    def gd_run(nsteps, x, g, host_obs=None):
        """Gradient descent: the image by the 1 / L step, the gains by their
        diagonal Newton step (per antenna and channel, the curvature is the
        sum over its baselines of |g V_pred|^2), damped by one half and
        capped at 0.05 per step."""
        losses = []
        for _ in range(nsteps):
            o = obs
            if host_obs is not None:
                o = host_obs.to(device, non_blocking=True)
            x.grad = None
            g.grad = None
            v = predict(x, plan)
            loss = (apply_gains(v, g, a1, a2) - o).abs().pow(2).sum()
            loss.backward()
            with torch.no_grad():
                x -= lr_x * x.grad
                pw = v.detach().abs().pow(2).sum(-1).double()  # [rows, chan]
                h = torch.zeros((nants, C), dtype=torch.float64, device=device)
                h.index_add_(0, a1l, pw)
                h.index_add_(0, a2l, pw)
                step = g.grad / (4.0 * h.clamp_min(1e-30))
                # at most 0.05 per step: while the image is far from the sky the
                # gains must not absorb its error
                step *= (0.05 / step.abs().clamp_min(0.05))
                g -= step
            losses.append(loss.detach())
        return losses

    def fresh():
        x = torch.zeros((1, npix, npix), dtype=torch.float32, device=device, requires_grad=True)
        g = torch.ones((nants, C), dtype=torch.complex128, device=device, requires_grad=True)
        return x, g

    x, g = fresh()
    gd_run(args.warmup, x, g)  # warm-up (plan caches, cuFFT)
    x, g = fresh()
    sampler = ClockSampler(device.index)
    _lib.profile_reset()
    _lib.profile_enable(True)
    sampler.start()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    losses = gd_run(args.gd_steps, x, g)
    b.record()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    _lib.profile_enable(False)
    stats = _lib.profile_read()
    ms = a.elapsed_time(b) / args.gd_steps
    losses = [float(v) for v in losses]
    img_err = float(numpy.linalg.norm(x.detach()[0].double().cpu().numpy() - sky) /
                    numpy.linalg.norm(sky))
    roof, kernels = roofline(stats, load_peaks())
    launches = sum(v["launches"] for k, v in stats.items() if not k.startswith("cufft"))
    # checks at this size: the dot-product identity through the Function
    xr = torch.randn((1, npix, npix), device=device, dtype=torch.float32, requires_grad=True)
    yr = torch.view_as_complex(torch.randn((R, C, 1, 2), device=device)).contiguous()
    vr = predict(xr, plan)
    lhs = torch.real(torch.vdot(yr.reshape(-1).to(torch.complex128),
                                vr.reshape(-1).to(torch.complex128)))
    lhs.backward()
    rhs = (xr.detach().double() * xr.grad.double()).sum()
    dot = abs(float(lhs) - float(rhs)) / float(
        torch.linalg.vector_norm(vr.detach().to(torch.complex128)) *
        torch.linalg.vector_norm(yr.to(torch.complex128)))
    # end to end: V_obs copied from page-locked host memory each step, loss read back
    host_obs = torch.empty(obs.shape, dtype=obs.dtype, pin_memory=True)
    host_obs.copy_(obs)
    x2, g2 = fresh()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ls = gd_run(args.e2e_gd_steps, x2, g2, host_obs)
    [float(v) for v in ls]
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.e2e_gd_steps
    # CPU baseline: one gradient step's dirty2ms + ms2dirty on the oracle's C
    # gridder, sampled over w-planes and scaled (host only)
    from oracle import cgridder
    cores = cgridder.max_threads()
    fun = uvw.reshape(-1, 3) * numpy.array([-1.0, 1.0, -1.0])
    s_ = freq / 299792458.0
    uu, vv, ww = [(fun[:, i:i + 1] * s_).ravel() for i in range(3)]
    rng2 = numpy.random.default_rng(2)
    dt, cplan, planes, nitems, t_cpu = cpu_gridder_sample(
        uu, vv, ww, lambda idx: rng2.standard_normal(idx.size) + 1j * rng2.standard_normal(
            idx.size), sky, npix, cell, eps, args.cpu_planes, 2.0, cores)
    plan.close()
    workload = {"workload": "differentiable predict: %d^2 FP32 sky (200 points + 20 Gaussian "
                            "blobs), %d antennas (%d baselines) x %d times, %d chan %.0f-%.0f "
                            "MHz, Stokes I, per-antenna gains, eps %g, %d GD steps"
                            % (npix, nants, nbl, nt, C, freq[0] / 1e6, freq[-1] / 1e6, eps,
                               args.gd_steps),
                "nvis": nvis, "l2": "plane batches and visibilities larger than L2"}
    step_vis = 2 * nvis  # one predict forward + one gridder backward per step
    return _aux_line(args, "Mvis/s gradient-descent steps (predict forward + adjoint backward) "
                     "on 1 GB300", step_vis / (ms * 1e-3) / 1e6, "Mvis/s", ms, workload, roof,
                     kernels, clocks, int(launches / args.gd_steps), dtype="f32",
                     steps=args.gd_steps,
                     gd={"steps": args.gd_steps, "ms_per_step": round(ms, 3),
                         "loss_first": losses[0], "loss_last": losses[-1],
                         "image_rel_err_last": img_err,
                         "obs_dft_s": round(t_dft, 2), "obs_components": int(len(ix))},
                     checks={"dot_product_rel_to_cauchy_schwarz": dot},
                     step_sizes={"image": lr_x, "lambda_max_AhA": lam,
                                 "gains": "diagonal Newton, damped by 1/2, at most 0.05 a step"},
                     cpu_baseline={"value": round(step_vis / t_cpu / 1e6, 4), "unit": "Mvis/s",
                                   "cores": cores, "kind": "port",
                                   "sample": "oracle C gridder (FP64), dirty2ms + ms2dirty of "
                                             "one step over %d of %d w-planes (%d items), "
                                             "scaled: %.2f s measured"
                                             % (len(planes), cplan.nplanes, nitems, dt)},
                     e2e={"value": round(step_vis / e2e_s / 1e6, 3), "unit": "Mvis/s",
                          "h2d_bytes_per_step": int(obs.numel() * 8), "d2h_bytes_per_step": 8,
                          "s_per_step": round(e2e_s, 4), "steps": args.e2e_gd_steps,
                          "api": "rascil_gb300.autograd.predict + apply_gains, torch autograd; "
                                 "V_obs from page-locked host memory each step, loss read back"})


def bench_dft(args):
    """The component DFT (dft_skycomponent_visibility) against the
    reference's own CUDA DFT kernel on the same GPU and inputs: LOW-like
    geometry, 2 hour angles x 130,816 baselines x 16 channels x 4 linear
    pols, 1,000 components, FP64 in both.  The reference kernel is the
    source string of rascil/processing_components/imaging/dft.py:181-258,
    built by oracle/ref_dft (its timing is this path's reference arm)."""
    import torch
    from rascil_gb300 import _lib
    from rascil_gb300 import simulation as sim
    from rascil_gb300.dft import dft_components
    device = torch.device("cuda", torch.cuda.current_device())
    _lib.load()
    uvw, freq, pc, cfg = sim.observation("low-like", ntimes=2)
    src = sim.sources(cfg)
    lmn = sim.lmn_rows(src)
    flux = sim.component_fluxes(cfg, src, len(freq))
    u = torch.from_numpy(uvw.reshape(-1, 3).copy()).to(device)
    f = torch.from_numpy(freq.copy()).to(device)
    nvis = uvw.shape[0] * uvw.shape[1] * len(freq) * flux.shape[-1]
    sampler = ClockSampler(device.index)
    ms, clocks, stats = _event_loop(
        lambda: dft_components(u, f, lmn, flux, precision="fp64", exact=True), args.steps,
        args.warmup, sampler)
    ms_fast, _, _ = _event_loop(
        lambda: dft_components(u, f, lmn, flux, precision="fp32", exact=False), args.steps,
        args.warmup, profile=False)
    ours = dft_components(u, f, lmn, flux, precision="fp64", exact=True).cpu().numpy()
    ref_line = {"unavailable": "the reference kernel was not built (oracle/ref_dft)"}
    try:
        from oracle import ref_dft
        uvw_lambda = (torch.from_numpy(uvw).to(device)[:, :, None, :]
                      * (f / 299792458.0)[None, None, :, None]).contiguous()
        lmn_t = torch.from_numpy(lmn).to(device).contiguous()
        flux_t = torch.from_numpy(flux).to(device).contiguous()
        ref = torch.zeros(uvw.shape[:2] + (len(freq), flux.shape[-1]), dtype=torch.complex128,
                          device=device)
        ms_ref, _, _ = _event_loop(lambda: ref_dft.run(lmn_t, flux_t, uvw_lambda, ref),
                                   args.steps, args.warmup, profile=False)
        b_ = ref.cpu().numpy().reshape(ours.shape)
        ref_line = {"value": round(nvis / (ms_ref * 1e-3) / 1e6, 3), "unit": "Mvis/s",
                    "ms": round(ms_ref, 3), "speedup_exact": round(ms_ref / ms, 3),
                    "speedup_fast": round(ms_ref / ms_fast, 3),
                    "max_rel_diff_exact": float(numpy.max(numpy.abs(ours - b_)) /
                                                numpy.max(numpy.abs(b_))),
                    "kind": "the reference's own CUDA dft_kernel (dft.py:181-258), same GPU"}
    except (ImportError, OSError, RuntimeError) as e:
        ref_line = {"unavailable": str(e)}
    # CPU baseline: the oracle's looped DFT (dft_cpu_looped restated) on the
    # first rows
    from oracle import dft as odft
    rs = 256
    ul = uvw.reshape(-1, 3)[:rs][None, :, None, :] * (freq / odft.SPEED_OF_LIGHT)[None, None, :,
                                                                                   None]
    t0 = time.perf_counter()
    odft.dft_cpu_looped(lmn, ul, flux)
    cpu_dt = time.perf_counter() - t0
    roof, kernels = roofline(stats, load_peaks())
    workload = {"workload": "component DFT: LOW-like geometry, 2 times x %d baselines x %d chan "
                            "x %d pols, %d components, FP64" % (uvw.shape[1], len(freq),
                                                               flux.shape[-1], len(lmn)),
                "nvis": nvis, "components": len(lmn)}
    return _aux_line(args, "Mvis/s component DFT (FP64, 1000 components) on 1 GB300",
                     nvis / (ms * 1e-3) / 1e6, "Mvis/s", ms, workload, roof, kernels, clocks, 1,
                     dtype="f64", fast_form={"ms": round(ms_fast, 3),
                                             "value": round(nvis / (ms_fast * 1e-3) / 1e6, 3)},
                     reference_kernel=ref_line,
                     cpu_baseline={"value": round(rs * len(freq) * flux.shape[-1] / cpu_dt / 1e6,
                                                  4), "unit": "Mvis/s", "cores": 1,
                                   "kind": "port", "sample": "oracle dft_cpu_looped (numpy) on "
                                   "the first %d rows: %.2f s" % (rs, cpu_dt)},
                     e2e=None)


def bench_batch(args):
    """The batched configuration: 256 independent snapshots (32-512 antennas
    in a 1 km disk, 1-8 channels in 100-200 MHz, 1-16 hour angles, 5e3-2e6
    Stokes I complex64 visibilities each, image side 256-2048, cell 1/(2.2
    max|uv|), epsilon 1e-5), invert + predict of every snapshot on device
    buffers.  Timed with CUDA events: the batch as one device program
    (SnapshotBatch), against one plan and call sequence per snapshot on one
    stream (plan creation included in both); the CPU oracle on a sample of
    snapshots, scaled by visibility count."""
    import torch
    from rascil_gb300 import _lib
    from rascil_gb300 import simulation as sim
    from rascil_gb300.batch import SnapshotBatch
    from rascil_gb300.wgridder import Plan
    device = torch.device("cuda", torch.cuda.current_device())
    _lib.load()
    raw = sim.snapshot_batch(args.nsnap)
    g = torch.Generator(device=device)
    g.manual_seed(1)
    snaps, vis, models = [], [], []
    for r in raw:
        u = torch.from_numpy(r["uvw"].reshape(-1, 3) * numpy.array([-1.0, 1.0, -1.0])).to(device)
        f = torch.from_numpy(r["freq"].copy()).to(device)
        snaps.append(dict(uvw=u, freq=f, npix=r["npix"], cell=r["cell"]))
        shape = (u.shape[0], f.shape[0], 1, 2)
        vis.append(torch.view_as_complex(torch.randn(shape, generator=g, device=device))
                   .contiguous())
        m = torch.zeros((1, r["npix"], r["npix"]), device=device)
        m[0, r["npix"] // 2, r["npix"] // 2 + 3] = 1.0
        models.append(m)
    nvis = sum(r["nvis"] for r in raw)
    eps = 1e-5

    def one_by_one(sigma):
        for i, sn in enumerate(snaps):
            p = Plan(sn["uvw"], sn["freq"], sn["npix"], sn["npix"], sn["cell"], sn["cell"], eps,
                     True, precision="fp32", grid_budget_bytes=2 << 30, sigma=sigma)
            p.ms2dirty(vis[i], layout="yx")
            p.dirty2ms(models[i], layout="yx")
            p.close()

    t0 = time.perf_counter()
    b = SnapshotBatch(snaps, eps, precision="fp32", nslots=args.nslots)
    torch.cuda.synchronize()
    plan_s = time.perf_counter() - t0
    sigmas = sorted({p.info["sigma"] for p in b.plans})
    sampler = ClockSampler(device.index)
    # the device program: per round one persistent gridding and one degridding
    # launch over every slot's snapshot (device work queue)
    ms_batch, clocks, stats = _event_loop(lambda: b.run_native(vis, models), args.steps,
                                          args.warmup, sampler)
    ms_loop, _, _ = _event_loop(lambda: b.run(vis, models), args.steps, 1, profile=False)
    b.capture(vis, models)
    ms_graph, _, _ = _event_loop(b.replay, args.steps, 1, profile=False)
    b.close()
    ms_seq, _, _ = _event_loop(lambda: one_by_one(0.0), 1, 1, profile=False)
    ms_seq2, _, _ = _event_loop(lambda: one_by_one(2.0), 1, 1, profile=False)
    launches = sum(v["launches"] for k, v in stats.items() if not k.startswith("cufft"))
    roof, kernels = roofline(stats, load_peaks())
    rate = lambda ms: round(2 * nvis / (ms * 1e-3) / 1e6, 2)  # noqa: E731
    # CPU baseline: the oracle's C gridder on a sample of snapshots (host only)
    from oracle import cgridder
    rng = numpy.random.default_rng(1)
    idx = rng.choice(len(raw), size=min(6, len(raw)), replace=False)
    cpu_t, cpu_v = 0.0, 0
    for i in idx:
        r = raw[i]
        uvw = r["uvw"].reshape(-1, 3) * numpy.array([-1.0, 1.0, -1.0])
        ms_ = rng.standard_normal((uvw.shape[0], len(r["freq"]))) * (1 + 0j)
        t0 = time.perf_counter()
        cgridder.ms2dirty(uvw, r["freq"], ms_, None, r["npix"], r["npix"], r["cell"], r["cell"],
                          eps, True)
        img = numpy.zeros((r["npix"], r["npix"]))
        img[r["npix"] // 2 + 3, r["npix"] // 2] = 1.0
        cgridder.dirty2ms(uvw, r["freq"], img, None, r["cell"], r["cell"], eps, True)
        cpu_t += time.perf_counter() - t0
        cpu_v += r["nvis"]
    workload = {"workload": "%d snapshots (32-512 antennas in 1 km, 1-8 chan in 100-200 MHz, "
                            "1-16 times, 256-2048 px, cell 1/(2.2 max|uv|)), eps 1e-5, FP32 "
                            "form, Stokes I, invert + predict" % len(raw),
                "nvis": int(nvis), "snapshots": len(raw),
                "image_sides": sorted(set(r["npix"] for r in raw))}
    return _aux_line(args, "Mvis/s invert+predict over 256 uneven snapshots on 1 GB300",
                     2 * nvis / (ms_batch * 1e-3) / 1e6, "Mvis/s", ms_batch, workload, roof,
                     kernels, clocks, int(launches / args.steps), dtype="f32",
                     program="gb_batch_run: pre-planned snapshots on %d slots, per round one "
                             "persistent gridding and one degridding launch over every slot's "
                             "snapshot (device work queue), transforms on the slot streams"
                             % args.nslots,
                     planner_sigmas=sigmas, plan_creation_s=round(plan_s, 3),
                     graph_replay={"ms": round(ms_graph, 1), "value": rate(ms_graph)},
                     per_snapshot_calls_on_slot_streams={"ms": round(ms_loop, 1),
                                                         "value": rate(ms_loop)},
                     one_plan_per_snapshot={"ms": round(ms_seq, 1), "value": rate(ms_seq),
                                            "note": "plan + invert + predict per snapshot on "
                                                    "one stream, planner's oversampling, plan "
                                                    "creation included"},
                     one_plan_per_snapshot_sigma2={"ms": round(ms_seq2, 1),
                                                   "value": rate(ms_seq2)},
                     cpu_baseline={"value": round(2 * cpu_v / cpu_t / 1e6, 4), "unit": "Mvis/s",
                                   "cores": cgridder.max_threads(), "kind": "port",
                                   "sample": "oracle C gridder (FP64) invert + predict of %d "
                                             "snapshots (%d vis): %.1f s" % (len(idx), cpu_v,
                                                                           cpu_t)},
                     e2e=None)


AUX_PATHS = {"weights": bench_weights, "rotation": bench_rotation, "lists": bench_lists,
             "autograd": bench_autograd, "dft": bench_dft, "batch": bench_batch}


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
    """The reference path's CPU stand-in, timed on the host cores: the oracle's
    C gridder (ducc0, the reference's gridder, cannot be installed here).
    Host only: the workload is built with numpy and the GPU library is never
    loaded.  Each step is one bounded sample (a few w-planes of one
    polarisation); the line's value extrapolates the measured sample time to
    the whole step, and says so."""
    rank, world = dist_setup(args)
    if rank != 0:
        return None
    cw = CpuWorkload(args.config, args.scale)
    samples = []
    for i in range(args.warmup + args.steps):
        r = cpu_sample(cw, args.ref_planes, nplanes_probe=1)
        if i >= args.warmup:
            samples.append(r)
    t_sample = float(numpy.mean([r["sample_s"] for r in samples]))
    t_full = float(numpy.mean([r["full_s"] for r in samples]))
    value = 2 * cw.nvis / t_full / 1e6
    r = samples[-1]
    rc = reduced_case(args.config)
    acc = cpu_accuracy(rc, r["sigma"], r["cores"])
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mvis/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t_sample * 1e3, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": workload_config(cw),
            "extrapolated": {"value_is_extrapolated": True,
                             "sample_s_measured": round(t_sample, 3),
                             "scale_to_full_step": round(r["scale"], 3),
                             "full_step_s_estimated": round(t_full, 1),
                             "how": "each step times one sample (%d of %d w-planes, one "
                                    "polarisation); value = 2 nvis / (sample s x %d/%d planes "
                                    "x %d pols); ms_per_step is the measured sample"
                                    % (r["planes"], r["nplanes"], r["nplanes"], r["planes"],
                                       cw.npol)},
            "accuracy_reduced_case": {"case": rc["desc"], "epsilon": rc["eps"], "cpu": acc},
            "cpu_baseline": {"value": round(value, 4), "unit": "Mvis/s", "cores": r["cores"],
                             "kind": "port", "sample": r["desc"]},
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


# What bounds each kernel of the step (ncu summaries under profiles/).
KERNEL_BOUND = {
    "k_grid": "shared-memory pipe (atomics and the sub-grid flush) and instruction issue "
              "(update rate in roofline.secondary)",
    "k_degrid": "L1 data pipe: grid rows read through L1, plus the item cache in shared memory "
                "(update rate in roofline.secondary)",
    "k_rows_forward": "instruction issue (DRAM traffic = algorithmic bytes)",
    "k_rows_inverse": "instruction issue (DRAM traffic = algorithmic bytes)",
    "k_col_a_inv": "hbm", "k_col_b_inv": "hbm", "k_col_b_pred": "hbm",
    "k_col_a_pred": "hbm", "grid_zero": "hbm (write only)",
}


def mid_like_run(args, device):
    """The MID-like configuration (197 dishes to 80 km, dec -60, 64 channels
    over 0.95-1.67 GHz, 4 pols, 512 times, 16384^2 image): 1 warm-up + a
    few timed FP32 steps, with the FP32 accuracy against the FP64 DFT."""
    import torch
    GRID = GRID_BUDGET[0]
    GRID_BUDGET[0] = int(40 * (1 << 30))  # one 32768^2 x 4-pol plane per batch
    try:
        wl = Workload("mid-like", "full", device)
        ms, out, _, _ = time_steps(wl, "fp32", wl.vis32, wl.wgt32, wl.model32, args.mid_steps,
                                   args.mid_warmup)
        dirty, pred, info = out
        acc = accuracy(wl, dirty, pred, "fp32")
        del dirty, pred, out
        res = {"value": round(2 * wl.nvis / (ms * 1e-3) / 1e6, 3), "unit": "Mvis/s",
               "ms_per_step": round(ms, 1), "steps": args.mid_steps, "warmup": args.mid_warmup,
               "config": workload_config(wl), "accuracy_fp32": acc,
               "plan": {k: info[k] for k in ("support", "sigma", "ngrid_x", "nplanes",
                                             "planes_per_batch", "fft_mode", "own_rows")}}
        del wl
    finally:
        GRID_BUDGET[0] = GRID
        torch.cuda.empty_cache()
    return res


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
    cw = CpuWorkload(args.config, args.scale)
    wl = Workload(args.config, args.scale, device, cpu=cw)
    sampler = ClockSampler(device.index) if rank == 0 else None
    tuned = tune(wl, "fp32", wl.vis32, wl.wgt32, wl.model32, args.tune_seconds) \
        if args.tune and not args.no_tune else None
    if world > 1:
        torch.distributed.barrier()
    ms, out, clocks, stats = time_steps(wl, "fp32", wl.vis32, wl.wgt32, wl.model32, args.steps,
                                        args.warmup, sampler=sampler, profile=True)
    ms = max_over_ranks(ms, world)
    dirty, pred, info = out
    value = world * 2 * wl.nvis / (ms * 1e-3) / 1e6
    acc32 = accuracy(wl, dirty, pred, "fp32")
    del dirty, pred, out
    smem = _lib.smem_peaks(_ptr_stream(torch.cuda.current_stream(device)))
    roof, kernels = roofline(stats, load_peaks(), smem)
    for k, b in KERNEL_BOUND.items():
        if k in kernels:
            kernels[k]["bound"] = b
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
            "smem_peaks": {"atomics_per_s": smem[0], "loads8_per_s": smem[1]},
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
    cpu_sigma = None
    if not args.no_cpu and rank == 0:
        # host only: a failure of the CPU gridder is reported in the line and
        # does not abort the GPU measurement (no device work in this block)
        try:
            r = cpu_sample(cw, args.cpu_planes, nplanes_probe=1)
            line["cpu_baseline"] = {"value": round(r["mvis"], 4), "unit": "Mvis/s",
                                    "cores": r["cores"], "kind": "port", "sample": r["desc"]}
            cpu_sigma = r["sigma"]
        except (OSError, ValueError, IndexError, MemoryError) as e:
            line["cpu_baseline"] = {"value": None, "unit": "Mvis/s", "cores": None,
                                    "kind": "port", "sample": "failed: %s" % e}
    del wl
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_reduced:
        # every form's error on one reduced case at the same epsilon, the CPU
        # path (the reference's stand-in) beside the GPU forms
        rc = reduced_case(args.config)
        red = {"case": rc["desc"], "epsilon": rc["eps"],
               "gpu_fp32": gpu_accuracy(rc, "fp32", device),
               "gpu_fp64": gpu_accuracy(rc, "fp64", device)}
        if not args.no_cpu:
            from oracle import cgridder
            red["cpu"] = cpu_accuracy(rc, cpu_sigma or 2.0, cgridder.max_threads())
        line["accuracy_reduced_case"] = red
    if rank == 0 and not args.no_mid:
        line["mid_like"] = mid_like_run(args, device)
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
