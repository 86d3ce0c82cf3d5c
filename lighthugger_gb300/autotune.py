"""Autotuner of the launch shape: raster bin thresholds and the schedule.

The raster kernels split triangles into three bins by the pixel count of
their bounding box -- rasterised by one lane (<= small_px), by one warp
(<= medium_px), or cut into chunks of 16 x 32 (visibility) or 16 x 64
(shadow) pixels spread over all warps --,
claim `raster_batch` meshlets per atomic, and a batched frame can run per
stage or as one persistent launch.  None of this
changes a single output bit; it only moves time.  `tune()` times frames of
the given workload with CUDA events for every candidate and keeps the
fastest; results are cached per GPU name and workload signature in
lighthugger_gb300/_build/tuning.json.
"""
import itertools
import json
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(_HERE, "_build", "tuning.json")

SMALL = (4, 8, 16, 32)
MEDIUM = (64, 128, 256, 512, 1024)
BATCH = (1, 2, 4, 8)


def _signature(renderer, n_probes, batched):
    import torch
    c = renderer.config
    return "%s|%dx%d|s%d|p%d|%s" % (torch.cuda.get_device_name(), c.width, c.height, c.shadow_size, n_probes,
                                    "batched" if batched else "plain")


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def _save(cache):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def time_frames(renderer, run, frames, stream):
    """Mean device milliseconds of `frames` calls of run() on `stream`."""
    import torch
    for _ in range(2):
        run()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        a.record(stream)
    for _ in range(frames):
        run()
    with torch.cuda.stream(stream):
        b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / frames


def tune(renderer, uniforms, probes=None, n_probes=0, batched=False, frames=4, use_cache=True, stream=None):
    """Pick and apply the fastest tuning for this workload; returns
    (tuning dict, {candidate: ms})."""
    import torch
    from . import SCHEDULE_PER_STAGE, SCHEDULE_PERSISTENT
    key = _signature(renderer, n_probes, batched)
    cache = _load() if use_cache else {}
    if key in cache:
        best = cache[key]
        renderer.set_tuning(small_px=best["small_px"], medium_px=best["medium_px"], schedule=best["schedule"],
                            raster_batch=best.get("raster_batch", 0))
        return best, {}
    stream = stream or torch.cuda.Stream()
    sptr = stream.cuda_stream
    if batched:
        run = lambda: renderer.frame_graph(uniforms, probes, n_probes, stream=sptr)
        schedules = (SCHEDULE_PER_STAGE, SCHEDULE_PERSISTENT)
    else:
        run = lambda: renderer.frame_graph(uniforms, None, 0, stream=sptr)
        schedules = (SCHEDULE_PER_STAGE,)
    results = {}
    best, best_ms = None, float("inf")
    # bins and schedule first (automatic claim batch), then the claim batch
    for sched, small, medium in itertools.product(schedules, SMALL, MEDIUM):
        if medium < small:
            continue
        renderer.set_tuning(small_px=small, medium_px=medium, schedule=sched, raster_batch=0)
        ms = time_frames(renderer, run, frames, stream)
        results["%d/%d/%d/0" % (sched, small, medium)] = ms
        if ms < best_ms:
            best_ms, best = ms, {"small_px": small, "medium_px": medium, "schedule": sched, "raster_batch": 0, "ms": ms}
    for batch in BATCH:
        renderer.set_tuning(small_px=best["small_px"], medium_px=best["medium_px"], schedule=best["schedule"],
                            raster_batch=batch)
        ms = time_frames(renderer, run, frames, stream)
        results["%d/%d/%d/%d" % (best["schedule"], best["small_px"], best["medium_px"], batch)] = ms
        if ms < best_ms:
            best_ms = ms
            best = dict(best, raster_batch=batch, ms=ms)
    renderer.set_tuning(small_px=best["small_px"], medium_px=best["medium_px"], schedule=best["schedule"],
                        raster_batch=best["raster_batch"])
    if use_cache:
        cache[key] = best
        _save(cache)
    return best, results
