"""Per-shape autotuner for a plan's free parameters.

The planner's free parameters -- grid oversampling ``sigma`` (with the
support W it implies for the requested epsilon), the uv tile side and the
number of w-planes per bucket slab -- trade FFT volume (about sigma^3 with
w-stacking), cuFFT efficiency (powers of two are much cheaper per point),
gridding work (about W^3) and bucket counts against each other, so the
best choice depends on the problem's shape.

:func:`autotune` times each candidate on the caller's real problem (one
plan + invert + predict, CUDA events on the current stream), keeps the
fastest, and caches it in memory and in a JSON file keyed by the shape
(``RASCIL_GB300_TUNING`` or ``~/.cache/rascil_gb300/tuning.json``).
:func:`choose` returns the cached choice for a shape, else a rule-based
default; :class:`rascil_gb300.wgridder.Plan` calls it whenever the caller
leaves sigma, tile and slab at 0.  ducc0 makes the same kind of choice
internally from a cost model; here it is measured.
"""
import json
import os
import threading

CANDIDATES = (
    {"sigma": 2.0, "tile": 32, "slab": 4},
    {"sigma": 2.0, "tile": 16, "slab": 2},
    {"sigma": 1.5, "tile": 16, "slab": 2},
    {"sigma": 1.5, "tile": 32, "slab": 2},
    {"sigma": 1.75, "tile": 16, "slab": 2},
)

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
    """Rule-based choice for shapes never tuned: sigma 2 (power-of-two grids
    for power-of-two images), 32-cell tiles, 4-plane slabs."""
    return {"sigma": 2.0, "tile": 32, "slab": 4}


def choose(key, npix_x, npix_y, nrows, nchan):
    with _lock:
        _load()
        hit = _mem.get(key)
    if hit:
        return {"sigma": hit["sigma"], "tile": hit["tile"], "slab": hit["slab"]}
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


def autotune(key, run, candidates=CANDIDATES, repeats=1):
    """Time ``run(params)`` (one plan + invert + predict) for every candidate,
    record and return the fastest.  Candidates the planner rejects (for
    example too many buckets) are skipped."""
    import torch
    timings = {}
    best, best_ms = None, None
    for cand in candidates:
        try:
            run(dict(cand))  # warm-up: cuFFT plans, caches
            torch.cuda.synchronize()
            start = torch.cuda.Event(enable_timing=True)
            stop = torch.cuda.Event(enable_timing=True)
            start.record()
            for _ in range(repeats):
                run(dict(cand))
            stop.record()
            torch.cuda.synchronize()
            ms = start.elapsed_time(stop) / repeats
        except ValueError:
            continue
        name = "sigma=%g,tile=%d,slab=%d" % (cand["sigma"], cand["tile"], cand["slab"])
        timings[name] = round(ms, 3)
        if best_ms is None or ms < best_ms:
            best, best_ms = dict(cand), ms
    if best is None:
        raise ValueError("no autotuning candidate is valid for this shape")
    record(key, best, timings)
    return best, timings
