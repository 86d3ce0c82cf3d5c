"""Autotuner of the launch shape (lh_tuning).

The knobs, none of which changes a single output bit (they only move time):

- occlusion_px: the two-pass occlusion raster's occluder threshold
  (projected sphere radius in pixels; 0 = one pass without occlusion test);
- small_px / medium_px: the raster's bins by bounding-box pixels -- one lane
  (<= small_px), one warp (<= medium_px; equal to small_px: no warp bin), or
  chunks spread over all warps;
- chunk_rows / chunk_cols: the chunk (tile) shape of big triangles, per pass
  (visibility, shadow);
- raster_batch: meshlets a raster warp claims per atomic;
- schedule: per stage or one persistent launch (batched frames);
- backward_rows: rows of a resolve-adjoint tile (tune_backward).

`tune()` times frames of the given workload with CUDA events and keeps the
fastest, one group of knobs at a time (coordinate descent from the current
tuning, groups in the order above); results are cached per GPU, target
sizes, scene (instances, triangles, seed) and camera (a hash of the
Uniforms) in lighthugger_gb300/_build/tuning.json.
"""
import hashlib
import json
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(_HERE, "_build", "tuning.json")

OCCLUSION = (0, 16, 32, 64, 128, 256, 512)
BINS = ((32, 32), (16, 16), (16, 64), (32, 64), (32, 128), (16, 128))  # (small_px, medium_px)
CHUNK = ((16, 32), (16, 64), (32, 64), (16, 128), (32, 128), (32, 256))  # (rows, columns)
BATCH = (0, 1, 2, 4)
BACKWARD_ROWS = (4, 8, 16)
KNOBS = ("small_px", "medium_px", "schedule", "raster_batch", "occlusion_px", "chunk_rows", "chunk_cols")


def signature(renderer, uniforms, n_probes, batched):
    """Cache key: GPU, target sizes, scene and camera of the workload."""
    import torch
    c = renderer.config
    d = renderer.scene.desc if getattr(renderer, "scene", None) is not None else None
    scene = "i%d|t%d|seed%d" % (d.n_instances, d.total_triangles, d.seed) if d is not None else "noscene"
    cam = hashlib.sha1(bytes(uniforms)).hexdigest()[:12]
    return "%s|%dx%d|s%d|p%d|%s|%s|cam%s" % (torch.cuda.get_device_name(), c.width, c.height, c.shadow_size,
                                            n_probes, "batched" if batched else "plain", scene, cam)


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def _save(cache, path):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


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


def _apply(renderer, t):
    renderer.set_tuning(**{k: t[k] for k in KNOBS})


def _label(t):
    return "occ%d/bins%d-%d/chunk%dx%d,%dx%d/batch%d/sched%d" % (
        t["occlusion_px"], t["small_px"], t["medium_px"], t["chunk_rows"][0], t["chunk_cols"][0], t["chunk_rows"][1],
        t["chunk_cols"][1], t["raster_batch"], t["schedule"])


def tune(renderer, uniforms, probes=None, n_probes=0, batched=False, frames=4, use_cache=True, stream=None,
         cache_path=None, digest=None):
    """Pick and apply the fastest tuning for this workload; returns
    (tuning dict with its "ms", {candidate label: ms}).  `digest`, if given,
    is called after each candidate's frames and its result stored per label
    in the returned results under "digests" (tests compare them)."""
    import torch
    from . import SCHEDULE_PER_STAGE, SCHEDULE_PERSISTENT
    path = cache_path or CACHE
    key = signature(renderer, uniforms, n_probes, batched)
    cache = _load(path) if use_cache else {}
    if key in cache:
        best = cache[key]
        _apply(renderer, best)
        return best, {}
    stream = stream or torch.cuda.Stream()
    sptr = stream.cuda_stream
    if batched:
        run = lambda: renderer.frame_graph(uniforms, probes, n_probes, stream=sptr)
        schedules = (SCHEDULE_PER_STAGE, SCHEDULE_PERSISTENT)
    else:
        run = lambda: renderer.frame_graph(uniforms, None, 0, stream=sptr)
        schedules = (SCHEDULE_PER_STAGE,)
    cur = renderer.tuning().as_dict()
    best = {k: cur[k] for k in KNOBS}
    results, digests = {}, {}
    best_ms = [float("inf")]

    def measure(cand):
        label = _label(cand)
        if label in results:
            return results[label]
        _apply(renderer, cand)
        ms = time_frames(renderer, run, frames, stream)
        results[label] = ms
        if digest is not None:
            digests[label] = digest()
        return ms

    def descend(options):
        nonlocal best
        for change in options:
            cand = dict(best, **change)
            ms = measure(cand)
            if ms < best_ms[0]:
                best_ms[0], best = ms, cand

    best_ms[0] = measure(best)
    descend({"occlusion_px": v} for v in OCCLUSION)
    descend({"small_px": a, "medium_px": b} for a, b in BINS)
    descend({"chunk_rows": [r, best["chunk_rows"][1]], "chunk_cols": [c, best["chunk_cols"][1]]} for r, c in CHUNK)
    descend({"chunk_rows": [best["chunk_rows"][0], r], "chunk_cols": [best["chunk_cols"][0], c]} for r, c in CHUNK)
    descend({"raster_batch": v} for v in BATCH)
    descend({"schedule": v} for v in schedules)
    _apply(renderer, best)
    best = dict(best, ms=best_ms[0])
    if use_cache:
        cache[key] = best
        _save(cache, path)
    if digest is not None:
        results["digests"] = digests
    return best, results


def tune_backward(renderer, grad_ptr, targets, frames=4, stream=None):
    """Pick and apply the fastest adjoint tile (backward_rows) for the last
    frame's resolve adjoint; returns (rows, {rows: ms})."""
    import ctypes as C
    import torch
    from . import _check, lib
    stream = stream or torch.cuda.Stream()
    sptr = stream.cuda_stream

    def run():
        _check(lib().lh_resolve_backward(renderer.ctx, grad_ptr, C.byref(targets), C.c_void_p(sptr)),
               "lh_resolve_backward", renderer.ctx)

    results = {}
    for rows in BACKWARD_ROWS:
        renderer.set_tuning(backward_rows=rows)
        results[rows] = time_frames(renderer, run, frames, stream)
    best = min(results, key=results.get)
    renderer.set_tuning(backward_rows=best)
    return best, results
