"""Per-shape autotuner for a plan's free parameters.

The planner's free parameters -- grid oversampling ``sigma`` (with the
support W it implies for the requested epsilon), the uv tile side, the
number of w-planes per bucket slab and the number of w-planes transformed
per batch -- trade FFT volume (about sigma^3 with w-stacking), transform
efficiency (the library's own pruned transforms need power-of-two grids
twice the image; other sizes use batched cuFFT plans), gridding work (about
W^3), bucket counts and batch memory against each other, so the best choice
depends on the problem's shape.

Without tuning, the planner picks sigma from its own cost model (as ducc0
does internally) and fixed tile / slab / batch rules.  :func:`autotune`
measures instead: starting from the planner's choice it varies one
parameter at a time over its options (sigma, then tile, slab and planes per
batch), times each candidate on the caller's real problem (one plan +
invert + predict, CUDA events on the current stream), keeps every
improvement, stops when the options are exhausted or its time budget is
spent, and caches the winner in memory and in a JSON file keyed by the
shape (``RASCIL_GB300_TUNING`` or ``~/.cache/rascil_gb300/tuning.json``).
:func:`choose` returns the cached choice for a shape, else all zeros (the
planner's own choice); :class:`rascil_gb300.wgridder.Plan` calls it
whenever the caller leaves sigma, tile, slab and planes per batch at 0.
"""
import json
import os
import threading
import time

SIGMAS = (2.0, 1.75, 1.5, 1.25)
TILES = (16, 32, 64)
SLABS = (2, 4, 8)
PARAMS = ("sigma", "tile", "slab", "planes")

_lock = threading.Lock()
_mem = {}
_loaded = [False]


def cache_path():
    p = os.environ.get("RASCIL_GB300_TUNING")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "rascil_gb300", "tuning.json")


def shape_key(npix_x, npix_y, pixsize_x, npol, precision, epsilon, do_wstacking, nrows, nchan):
    """Key of a tuning entry: image geometry, data volume and accuracy."""
    return "|".join(str(x) for x in (
        int(npix_x), int(npix_y), "%.6g" % float(pixsize_x), int(npol), precision,
        "%.3g" % float(epsilon), int(bool(do_wstacking)), int(nrows), int(nchan)))


def _load():
    if _loaded[0]:
        return
    _loaded[0] = True
    try:
        with open(cache_path()) as f:
            data = json.load(f)
        if isinstance(data, dict) and data.get("version") == 1:
            _mem.update({k: v for k, v in data.get("entries", {}).items()
                         if isinstance(v, dict) and "sigma" in v})
    except (OSError, ValueError):
        pass


def _save():
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump({"version": 1, "entries": _mem}, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def default_params(npix_x, npix_y, nrows, nchan):
    """For shapes never tuned: all zero, the planner's own choice -- the grid
    oversampling of least modelled cost (gridding work against per-plane
    transform work), 32-cell tiles (16 in the FP64 form), 4-plane slabs."""
    return {"sigma": 0.0, "tile": 0, "slab": 0}


def choose(key, npix_x, npix_y, nrows, nchan):
    with _lock:
        _load()
        hit = _mem.get(key)
    if hit:
        out = {"sigma": hit["sigma"], "tile": hit["tile"], "slab": hit["slab"]}
        if hit.get("planes"):
            out["planes"] = hit["planes"]
        return out
    return default_params(npix_x, npix_y, nrows, nchan)


def record(key, params, timings):
    with _lock:
        _load()
        _mem[key] = dict(params, timings=timings)
        _save()


def forget(key=None):
    """Drop one cached entry (or all) from memory and the file."""
    with _lock:
        _load()
        if key is None:
            _mem.clear()
        else:
            _mem.pop(key, None)
        _save()


def _name(c):
    return ",".join("%s=%g" % (k, c[k]) for k in PARAMS if k in c)


def _time(run, cand, repeats):
    import torch
    run(dict(cand))  # warm-up: cuFFT plans, caches
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(repeats):
        run(dict(cand))
    stop.record()
    torch.cuda.synchronize()
    return start.elapsed_time(stop) / repeats


def autotune(key, run, start=None, candidates=None, max_seconds=120.0, repeats=1,
             plane_bytes=None, max_batch_bytes=64 << 30):
    """Time candidates of ``run(params)`` (one plan + invert + predict with
    params sigma / tile / slab / planes), record and return the fastest with
    every timing.

    :param start: the planner's own choice (sigma, tile, slab, planes as a
        plan reported them); the search starts from it and varies one
        parameter at a time: sigma over SIGMAS, tile over TILES, slab over
        SLABS, planes per batch over half / double the start (kept below
        ``max_batch_bytes`` when ``plane_bytes``, one plane's grid bytes at
        the start's sigma, is given)
    :param candidates: an explicit list instead of the search
    :param max_seconds: tuning time budget; no new candidate starts after it
    Candidates the planner rejects (ValueError) are skipped."""
    t0 = time.perf_counter()
    timings = {}
    best, best_ms = None, None

    def consider(cand):
        nonlocal best, best_ms
        name = _name(cand)
        if name in timings or time.perf_counter() - t0 > max_seconds:
            return
        try:
            ms = _time(run, cand, repeats)
        except ValueError:
            timings[name] = None
            return
        timings[name] = round(ms, 3)
        if best_ms is None or ms < best_ms:
            best, best_ms = dict(cand), ms

    if candidates is not None:
        for cand in candidates:
            consider(dict(cand))
    else:
        if start is None:
            raise ValueError("autotune needs the planner's choice (start) or candidates")
        base = {k: start[k] for k in PARAMS}
        consider(base)
        options = {"sigma": SIGMAS, "tile": TILES, "slab": SLABS}
        pl = int(base["planes"])
        opts = [p for p in (max(1, pl // 2), 2 * pl) if p != pl]
        if plane_bytes:
            opts = [p for p in opts if p * plane_bytes <= max_batch_bytes]
        options["planes"] = tuple(opts)
        for k in PARAMS:
            centre = dict(best) if best else dict(base)
            for v in options[k]:
                if v == centre[k]:
                    continue
                cand = dict(centre)
                cand[k] = v
                if k == "sigma":
                    cand["planes"] = 0  # the batch follows the new grid size
                consider(cand)
    if best is None:
        raise ValueError("no autotuning candidate is valid for this shape")
    record(key, best, timings)
    return best, timings
