"""Autotuner for the raster kernel's launch shape.

Picks, for a renderer whose scenes are already populated, the CTA size
(threads), the batched form's region size (the screen tile one CTA owns),
the small-triangle threshold (bounding boxes up to this many pixels are
rasterised by one lane, larger ones by the whole CTA from the shared-memory
bin; 1 and 4 px with every shape, 8 and 16 px on the best), the bin
capacity in use (how full the bin gets before the CTA rasterises it) and
the per-scene form's region size.  Each candidate is timed with CUDA
events around the raster launch over a few draws of the caller's own poses;
the best is applied and cached in a JSON file keyed by GPU name and a
signature of the workload (scene count, resolutions, triangles), so a later
process with the same workload skips the search.
"""
import hashlib
import json
import os
import statistics

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "gbr_autotune.json")

# Launch shapes of the batched form: threads per CTA (8, 16 or 32 warps per
# region), CTAs per SM, the region (screen tile) one CTA owns -- from 128 x 128
# down to 32 x 32 -- and the small-triangle threshold.
BATCHED_SPACE = ([dict(threads=1024, region_width=rw, region_height=rh, small_area=sa, ctas_per_sm=1)
                  for (rw, rh) in ((128, 128), (128, 64), (64, 64)) for sa in (1, 4)] +
                 [dict(threads=512, region_width=rw, region_height=rh, small_area=sa, ctas_per_sm=2)
                  for (rw, rh) in ((128, 64), (64, 64)) for sa in (1, 4)] +
                 [dict(threads=256, region_width=rw, region_height=rh, small_area=sa, ctas_per_sm=4)
                  for (rw, rh) in ((64, 64), (32, 32)) for sa in (1, 4)])
# Larger small-triangle thresholds, tried on the best shape (sub-pixel scan
# geometry gains from 8 px, finer-grained scenes lose beyond 4).
SMALL_AREA = (8, 16)
# Bin capacity in use: the share of the shared triangle queue that triggers
# its rasterisation, tried on the best shape.
QUEUE_FILL = (50, 75, 100)
PLAIN_SPACE = [dict(plain_region_width=w, plain_region_height=h) for (w, h) in
               ((16, 32), (32, 32), (16, 16))]


def signature(renderer, triangles):
    n = renderer.sceneCount()
    sizes = sorted({renderer.sceneViewport(s)[2:] for s in range(n)})
    key = json.dumps([n, sizes, int(triangles)])
    return hashlib.sha256(key.encode()).hexdigest()[:16]


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:
        return "unknown"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _time_batched(renderer, poses, draws):
    import habitat_sim_gb300 as gb
    times = []
    for i in range(draws + 1):
        renderer.updateCameras(*poses[i % len(poses)])
        renderer.draw(mode=gb.DrawMode.Batched, graph=True)
        st = renderer.lastDrawStats()
        if i:
            times.append(st["raster_ms"])
    return statistics.median(times)


def _time_plain(renderer, poses, draws):
    import time

    import torch

    import habitat_sim_gb300 as gb
    times = []
    for i in range(draws + 1):
        renderer.updateCameras(*poses[i % len(poses)])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        renderer.draw(mode=gb.DrawMode.PerScene)
        torch.cuda.synchronize()
        if i:
            times.append((time.perf_counter() - t0) * 1e3)
    return statistics.median(times)


def tune(renderer, poses, triangles, cache=DEFAULT_CACHE, draws=2, plain=True, force=False):
    """Choose and apply the launch shape; returns (tuning dict, report dict)."""
    sig = f"{_gpu_name()}:{signature(renderer, triangles)}"
    data = _load(cache)
    if not force and sig in data:
        renderer.setTuning(**data[sig]["tuning"])
        return renderer.tuning(), {"cached": True, **data[sig]}
    renderer.setKernelTiming(True)
    trials = []
    for cand in BATCHED_SPACE:
        try:
            renderer.setTuning(**cand)
        except Exception as e:   # does not fit this GPU's shared memory
            trials.append(dict(cand, error=str(e)))
            continue
        trials.append(dict(cand, raster_ms=_time_batched(renderer, poses, draws)))
    best = min((t for t in trials if "raster_ms" in t), key=lambda t: t["raster_ms"])
    for sa in SMALL_AREA:
        cand = dict({k: best[k] for k in ("threads", "region_width", "region_height", "ctas_per_sm")},
                    small_area=sa)
        renderer.setTuning(**cand)
        t = dict(cand, raster_ms=_time_batched(renderer, poses, draws))
        trials.append(t)
        if t["raster_ms"] < best["raster_ms"]:
            best = t
    shape = {k: best[k] for k in ("threads", "region_width", "region_height", "small_area", "ctas_per_sm")}
    renderer.setTuning(**shape, queue_fill_percent=75)
    best = dict(best, queue_fill_percent=75)
    for fill in QUEUE_FILL:
        if fill == 75:
            continue
        renderer.setTuning(queue_fill_percent=fill)
        t = dict(shape, queue_fill_percent=fill, raster_ms=_time_batched(renderer, poses, draws))
        trials.append(t)
        if t["raster_ms"] < best["raster_ms"]:
            best = t
    renderer.setTuning(**shape, queue_fill_percent=best["queue_fill_percent"])
    plain_trials = []
    if plain:
        for cand in PLAIN_SPACE:
            renderer.setTuning(**cand)
            plain_trials.append(dict(cand, step_ms=_time_plain(renderer, poses, 1)))
        pbest = min(plain_trials, key=lambda t: t["step_ms"])
        renderer.setTuning(**{k: pbest[k] for k in ("plain_region_width", "plain_region_height")})
    tuning = renderer.tuning()
    entry = {"tuning": tuning, "trials": trials, "plain_trials": plain_trials}
    data[sig] = entry
    try:
        _store(cache, data)
    except OSError:
        pass
    return tuning, {"cached": False, **entry}
