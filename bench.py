"""Benchmark of the GB300 visibility pipeline (one JSON line on rank 0).

Workload: the plain large configuration -- 4,096 instances of 8 seeded
procedural meshes (~50M triangles before culling), 16 textured materials,
one 1920x1080 main view + 4 shadow cascades, full frame: instance cull +
prefix sum, meshlet cull, visibility raster, depth reduction, cascade fit,
shadow cull + raster, lighting resolve.  A step is one frame.

  value  device time of one frame replayed from the context's CUDA graph
         (lh_frame_graph; CUDA events on the frame's stream), L2 flushed
         between frames by writing a 256 MiB buffer (untimed); launch_ms is
         the same frame through lh_frame (13 launches with programmatic
         dependent launch between them)
  e2e    the same frame through the C ABI with host buffers: per-frame
         uniforms copied from pinned host memory and the HDR image read back
         to pinned host memory (lh_frame_readback: the copy of frame i
         overlaps frame i + 1's culling and rasterisation), wall clock over
         the steps; serial_value is one frame + readback at a time
  cpu_baseline  the CPU oracle (C++ restatement of the reference shaders) on
         the host cores, same scene, median of a few frames

`--impl reference` times the reference's CPU path instead: the reference is a
Vulkan renderer that cannot run here, so its shaders' CPU restatement (the
oracle) stands in for it, with every host thread.

Multi-GPU: the path does not shard (one view set per frame); under torchrun
each rank renders an independent replica and value is the frame time
(max over ranks).
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "1080p frame ms (cull+raster+resolve)"

# Algorithmic bytes per unit (per-stage rooflines).
INSTANCE_BYTES = 112
MESHLET_BYTES = 56
PREFIX_ENTRY_BYTES = 8
DRAW_WRITE_BYTES = 8 + 16
RASTER_DRAW_BYTES = 48       # the raster draw record written per visible meshlet, read by the raster
VIS_PIXEL_BYTES = 8
HDR_PIXEL_BYTES = 16
RASTER_TRI_BYTES = 3 + 0.52 * (4 + 12)  # micro indices + ~0.52 unique vertices (index + fp32 position)
FRAGMENT_BYTES = 8           # one 64-bit depth-test reduction per fragment
# Per-kernel DRAM bytes of the workload, from the committed ncu capture
# summary (profiles/dram_bytes_c2_frame.txt: command, commit, one line per
# kernel); `traffic` in the roofline is read from there, never measured here.
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "dram_bytes_c2_frame.txt")
# (k_raster_alpha<K> launches only for scenes with alpha-clip meshes)
STAGE_KERNELS = {
    "raster": ("k_raster<0, 3>", "k_raster_alpha<0>", "k_raster_big<0>", "k_hiz", "k_occlusion_filter"),
    "shadow_raster": ("k_raster<1, 3>", "k_raster_alpha<1>", "k_raster_big<1>"),
    "resolve": ("k_resolve<1>",),
    "cull_meshlets": ("k_cull_meshlets",),
    "depth_fit": ("k_depth_reduce_fit",),
}


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def _clock_sampler():
    """Sample SM clocks and throttle reasons during the timed region."""
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    try:
        return subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "200"],
                                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except Exception:
        return None


def _clock_summary(proc, gpu_index):
    if proc is None:
        return None
    try:
        proc.terminate()
        out, _ = proc.communicate(timeout=5)
    except Exception:
        return None
    sms, maxes, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in out.splitlines():
        f = [x.strip() for x in line.split(",")]
        if len(f) < 9 or f[0] != str(gpu_index):
            continue
        try:
            sms.append(float(f[1]))
            maxes.append(float(f[2]))
        except ValueError:
            continue
        for n, v in zip(names, f[5:9]):
            if v.lower() == "active":
                reasons.add(n)
    if not sms:
        return None
    sms.sort()
    return {"sm_mhz": sms[len(sms) // 2], "sm_max_mhz": max(maxes), "reasons": sorted(reasons), "samples": len(sms)}


def _measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(stage, alpha_scene=False):
    """DRAM bytes per frame of a stage's kernels from the committed capture
    summary, with the summary's provenance line; (None, None) if absent.
    The alpha-clip kernels count only for a scene with alpha-clip meshes."""
    try:
        with open(TRAFFIC_FILE) as f:
            lines = f.read().splitlines()
    except OSError:
        return None, None
    source = next((l[2:].strip() for l in lines if l.startswith("# capture:")), TRAFFIC_FILE)
    per = {}
    for l in lines:
        if not l.strip() or l.startswith("#"):
            continue
        name, rd, wr = l.rsplit(None, 2)
        per[name.strip()] = per.get(name.strip(), 0.0) + float(rd) + float(wr)  # kernels run twice add up
    names = [n for n in STAGE_KERNELS.get(stage, ()) if n in per and ("alpha" not in n or alpha_scene)]
    if not names:
        return None, None
    return sum(per[n] for n in names), "profiles/dram_bytes_c2_frame.txt: " + source


def atomic_peak(lh, torch, stream, mib=16, reps=16):
    """Reductions per second of the raster's depth-test instruction
    (lh_probe_red_u64) over a buffer the size of the visibility target, both
    patterns, best of 4, CUDA events on `stream`."""
    L = lh.lib()
    n = mib * 1024 * 1024 // 8
    buf = torch.zeros(n, dtype=torch.int64, device="cuda")
    out = {"buffer_mib": mib}
    for name, scattered in (("contiguous", 0), ("scattered", 1)):
        best = 0.0
        for _ in range(4):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                a.record(stream)
            lh._check(L.lh_probe_red_u64(buf.data_ptr(), n, scattered, reps, stream.cuda_stream), "lh_probe_red_u64")
            with torch.cuda.stream(stream):
                b.record(stream)
            torch.cuda.synchronize()
            best = max(best, n * reps / (a.elapsed_time(b) * 1e-3))
        out[name + "_per_s"] = best
    return out


def reduce_max_over_ranks(value, device=None):
    """Max of a per-rank float over the process group (identity with one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_oracle_frames(scene, frames, threads=0):
    from oracle import binding as ob
    d = scene.desc
    times, stages, fr = [], [], None
    for _ in range(frames):
        fr = ob.run_scene(scene, shadow_size=d.shadow_size, max_instances=max(1024, d.n_instances), threads=threads)
        times.append(fr.stage_ms["total"])
        stages.append(fr.stage_ms)
    n_threads = int(stages[-1]["threads"]) if stages else 0
    s = sorted(times)
    return s[len(s) // 2], n_threads, stages[-1] if stages else {}, fr


def hdr_error_vs_f64(gpu_hdr, fr):
    """The GPU image against the oracle's float64 resolve of the same
    visibility (and the oracle's own float32 image against it), over the
    covered pixels: max and 99th percentile of the absolute error."""
    import numpy as np
    from oracle import binding as ob
    h64 = ob.resolve_f64(fr)[..., :3]
    cov = (fr.vis >> np.uint64(32)) != 0
    out = {"pixels": int(cov.sum())}
    for name, img in (("gpu", gpu_hdr), ("oracle_f32", fr.hdr)):
        e = np.abs(img[..., :3].astype(np.float64) - h64)[cov]
        out[name + "_max_abs"] = float(e.max()) if e.size else 0.0
        out[name + "_p99_abs"] = float(np.percentile(e, 99)) if e.size else 0.0
    out["gpu_vs_oracle_f32_max_abs"] = float(np.abs(gpu_hdr[..., :3].astype(np.float64) -
                                                    fr.hdr[..., :3].astype(np.float64)).max())
    return out


def run_reference(args):
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    import lighthugger_gb300 as lh
    from oracle import binding as ob
    ob.lib()
    scene = lh.Scene(args.config, seed=args.seed)
    d = scene.desc
    for _ in range(args.warmup):
        ob.run_scene(scene, shadow_size=d.shadow_size, max_instances=max(1024, d.n_instances))
    times = []
    last = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        last = ob.run_scene(scene, shadow_size=d.shadow_size, max_instances=max(1024, d.n_instances))
        times.append((time.perf_counter() - t0) * 1e3)
    ms = sum(times) / len(times)
    threads = int(last.stage_ms["threads"])
    line = {
        "impl": "reference", "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": _workload_name(args.config, d), "seed": scene.seed},
        "cpu_baseline": {"value": ms, "unit": "ms", "cores": threads, "kind": "port",
                         "sample": "%d full frames of the workload on %d host threads" % (args.steps, threads)},
        "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "stage_ms": {k: round(v, 3) for k, v in last.stage_ms.items() if k not in ("threads",)},
    }
    print(json.dumps(line), flush=True)
    return 0


def _workload_name(cfg, d):
    names = {1: "plain-small", 2: "plain-large", 3: "batched-views", 4: "differentiable-resolve", 5: "stress"}
    return "%s: %d instances, %.1fM triangles before culling, %dx%d + 4 cascades %d^2" % (
        names.get(cfg, str(cfg)), d.n_instances, d.total_triangles / 1e6, d.width, d.height, d.shadow_size)


def _autotune(r, u, stream, args, probes=None, n_probes=0, frames=4):
    """The launch shape the autotuner picks for this workload (it times
    frames of each candidate before anything here is timed; no candidate
    changes a result bit): {"candidates": n, "tuning_ms": wall ms} or None."""
    if not args.tune:
        return None
    from lighthugger_gb300 import autotune
    t0 = time.perf_counter()
    _, results = autotune.tune(r, u, probes, n_probes, batched=n_probes > 0, frames=frames, use_cache=False,
                               stream=stream)
    return {"candidates": len(results), "tuning_ms": round((time.perf_counter() - t0) * 1e3, 1)}


def run_gpu(args):
    import numpy as np
    import torch
    import lighthugger_gb300 as lh
    from lighthugger_gb300 import build as native_build
    rank, world, local_rank = _env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    native_build.build()
    scene = lh.Scene(args.config, seed=args.seed).upload(local_rank)
    d = scene.desc
    cap = max(1024, d.n_instances)
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=cap, max_draws=2000000,
                    device=local_rank)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    u = scene.uniforms
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    tune_results = _autotune(r, u, stream, args, frames=10)
    for _ in range(max(3, args.warmup)):
        r.frame(u, stream=sptr)
    torch.cuda.synchronize()
    st = r.status()
    def timed_frames(run, steps):
        """Device ms of each frame (events on the frame stream), the 256 MiB
        flush written before each, outside the events."""
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                evs[i][0].record(stream)
            run()
            with torch.cuda.stream(stream):
                evs[i][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    clocks = _clock_sampler()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # the timed frames: lh_frame_graph, the frame's kernels replayed from the
    # context's CUDA graph (one launch: the device time cannot include the
    # host's enqueue of 13 kernels), no stage events inside them
    for _ in range(2):
        r.frame_graph(u, None, 0, stream=sptr)
    torch.cuda.synchronize()
    ms_steps = timed_frames(lambda: r.frame_graph(u, None, 0, stream=sptr), args.steps)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = _clock_summary(clocks, local_rank)
    ms = sum(ms_steps) / len(ms_steps)
    # per-stage split: the same frames again with an event between stages
    r.set_profiling(True)
    stage_acc = {k: 0.0 for k in lh.STAGES}
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        r.frame(u, stream=sptr)
        for k, v in r.stage_times().items():
            stage_acc[k] += v
    stage_ms = {k: v / args.steps for k, v in stage_acc.items()}
    r.set_profiling(False)
    # the same frame as individual launches (lh_frame; programmatic
    # dependent launch between its kernels); when the host enqueues slower
    # than the L2 flush runs, this includes the device waiting for it
    launch_steps = timed_frames(lambda: r.frame(u, stream=sptr), args.steps)
    launch_ms = sum(launch_steps) / len(launch_steps)
    ms = reduce_max_over_ranks(ms, device="cuda")

    # e2e through the C ABI with host buffers.  Pipelined (lh_frame_readback):
    # every frame sends its uniforms (560 bytes) and frame constants (8) to
    # the device as the replayed graph's frame-start kernel parameters, and
    # its HDR image is copied to one of two pinned host buffers while the next frame culls and
    # rasterises; wall clock over the steps, from an idle GPU to the last
    # image on the host.  Serial (lh_frame + lh_download, one frame at a
    # time) is reported beside it.
    npx = d.width * d.height
    host_hdr = [torch.empty(npx * 16, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
    for i in range(args.warmup):
        r.frame_readback(u, host_hdr[i & 1].data_ptr(), stream=sptr)
    r.readback_wait()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        r.frame_readback(u, host_hdr[i & 1].data_ptr(), stream=sptr)
    r.readback_wait()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = r.frame(u, stream=sptr)
        lh._check(lh.lib().lh_download(r.ctx, host_hdr[0].data_ptr(), out.hdr, npx * 16), "lh_download", r.ctx)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append((t1 - t0) * 1e3)
    e2e_serial_ms = sum(e2e_times) / len(e2e_times)

    # rooflines.  Algorithmic bytes per stage (the per-unit figures above
    # times this frame's units), over each stage's CUDA-event time
    st = r.status()
    vis_inst = st.visible_instances[0]
    cand = st.candidate_meshlets[0]
    vis_ml = st.visible_opaque[0] + st.visible_alpha_clip[0]
    cand_sh = sum(st.candidate_meshlets[1:5])
    vis_sh = sum(st.visible_opaque[1:5]) + sum(st.visible_alpha_clip[1:5])
    frag_main, frag_shadow = int(st.fragments[0]), int(st.fragments[1])
    # resolve: visibility words read, HDR written, plus what it gathers once:
    # the 4 shadow layers, the textures, and the geometry of the triangles
    # left in the visibility buffer (micro indices, ~0.52 unique vertices per
    # triangle of index + fp32 position / normal / uv)
    vis_ids = np.unique(r.visibility().reshape(-1) & np.uint64(0xFFFFFFFF))
    shown_tris = int(vis_ids.size)
    tex_bytes = sum(int(d.host_textures[i].width) * int(d.host_textures[i].height) * 4 for i in range(d.n_textures))
    tri_main, tri_shadow = visible_triangles(r, st, 0), sum(visible_triangles(r, st, v) for v in range(1, 5))
    algo = {
        "cull_instances": d.n_instances * INSTANCE_BYTES + vis_inst * PREFIX_ENTRY_BYTES,
        "cull_meshlets": cand * (MESHLET_BYTES + PREFIX_ENTRY_BYTES) + vis_ml * (DRAW_WRITE_BYTES + RASTER_DRAW_BYTES),
        "raster": int(tri_main * RASTER_TRI_BYTES) + frag_main * FRAGMENT_BYTES + vis_ml * RASTER_DRAW_BYTES,
        "depth_fit": npx * VIS_PIXEL_BYTES,
        "shadow_cull_meshlets": cand_sh * (MESHLET_BYTES + PREFIX_ENTRY_BYTES) +
        vis_sh * (DRAW_WRITE_BYTES + RASTER_DRAW_BYTES),
        "shadow_raster": int(tri_shadow * RASTER_TRI_BYTES) + frag_shadow * FRAGMENT_BYTES + vis_sh * RASTER_DRAW_BYTES,
        "resolve": npx * (VIS_PIXEL_BYTES + HDR_PIXEL_BYTES) + 4 * d.shadow_size ** 2 * 4 + tex_bytes +
        int(shown_tris * (3 + 0.52 * (4 + 32))),
    }
    peak, peak_kind = _measured_peak_hbm()
    per_stage = {}
    for k, b in algo.items():
        t = stage_ms.get(k, 0.0)
        if t > 0:
            gbs = b / (t * 1e-3) / 1e9
            per_stage[k] = {"ms": round(t, 4), "algorithmic_bytes": int(b), "achieved_gbs": round(gbs, 1),
                            "frac": round(gbs / peak, 4)}
    dom = max(algo, key=lambda k: stage_ms.get(k, 0.0))  # the dominant stage
    achieved = algo[dom] / (stage_ms[dom] * 1e-3) / 1e9
    traffic, traffic_src = (committed_traffic(dom, bool(scene.params.get("alpha_clip_materials")))
                            if args.config == 2 else (None, None))
    atom = atomic_peak(lh, torch, stream)
    red_rate = frag_main / (stage_ms["raster"] * 1e-3)
    tri_total = d.total_triangles
    tune = r.tuning()
    line = {
        "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scene, seed %d)" % scene.seed,
        "config": {"workload": _workload_name(args.config, d), "l2": "flushed between frames (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        # the visibility raster's rate over the triangles of the visible meshlets
        "gtri_per_s": tri_main / (stage_ms["raster"] * 1e-3) / 1e9,
        # the whole frame over the scene's triangles before culling
        "scene_gtri_per_s_before_culling": tri_total / (ms * 1e-3) / 1e9,
        "visible_meshlets": vis_ml, "candidate_meshlets": cand, "visible_instances": vis_inst,
        "shadow_visible_meshlets": [int(st.visible_opaque[k]) for k in range(1, 5)],
        "big_triangles_last_pass": int(st.big_triangles), "clipped_triangles_last_pass": int(st.clipped_triangles),
        "stage_ms": {k: round(v, 4) for k, v in stage_ms.items()},
        "launch_ms": launch_ms,
        "raster": {"visible_triangles": tri_main, "shadow_triangles": tri_shadow,
                   "fragments": frag_main, "shadow_fragments": frag_shadow,
                   "gtri_per_s": tri_main / (stage_ms["raster"] * 1e-3) / 1e9,
                   "shadow_gtri_per_s": tri_shadow / (stage_ms["shadow_raster"] * 1e-3) / 1e9,
                   "fragments_per_s": red_rate,
                   # fragments are 64-bit reductions: against the probe's ceiling
                   "atomic_frac_of_scattered_peak": red_rate / atom["scattered_per_s"],
                   "atomic_peak": atom},
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": 560 + 8, "d2h_bytes_per_step": npx * 16,
                "pipelined": True, "serial_value": e2e_serial_ms},
        # per frame: clear; 2 x (cull instances, cull meshlets, raster opaque,
        # raster alpha clip, chunks); depth + fit; resolve; with the occlusion
        # raster the visibility view adds the occluder pass, its chunks, the
        # hierarchical depth and the depth test of the other meshlets; the two
        # alpha-clip launches only when a mesh of the scene is alpha clip
        "gpu_launches": (13 + (4 if tune.occlusion_px else 0)
                         - (0 if scene.params.get("alpha_clip_materials") else 2)) * args.steps,
        "tuning": dict(tune.as_dict(), autotuned=tune_results),
        "occlusion": {"occluder_px": int(tune.occlusion_px), "occluders": int(st.occlusion[0]),
                      "survivors_opaque": int(st.occlusion[1]), "survivors_alpha": int(st.occlusion[2]),
                      "visible_opaque": int(st.visible_opaque[0])},
        "roofline": {"bound": "hbm", "kernel": dom + " stage (" + ", ".join(
                         k for k in STAGE_KERNELS.get(dom, (dom,))
                         if "alpha" not in k or scene.params.get("alpha_clip_materials")) + ")",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": (peak_kind + " (MEASURED_PEAKS.json hbm_gbs)") if peak_kind == "measured"
                     else peak_kind,
                     "traffic": traffic, "traffic_source": traffic_src, "algorithmic_bytes": int(algo[dom])},
        "per_stage_roofline": per_stage,
        "status_flags": int(st.flags),
    }
    if clk:
        line["clocks"] = clk
    if args.batched:
        line["batched"] = bench_batched(lh, torch, args, local_rank)
    if args.differentiable:
        line["differentiable"] = bench_differentiable(lh, torch, args, local_rank)
    if args.stress:
        line["stress"] = bench_stress(lh, torch, args, local_rank)
    if rank == 0 and args.cpu_frames > 0:
        gpu_hdr = r.hdr()
        med, threads, stages, fr = cpu_oracle_frames(scene, args.cpu_frames)
        line["cpu_baseline"] = {"value": med, "unit": "ms", "cores": threads, "kind": "port",
                                "sample": "median of %d full frames of the workload" % args.cpu_frames,
                                "speedup_vs_gpu_frame": med / ms}
        # the HDR's error against the float64 resolve of the same frame
        line["hdr_error_vs_f64"] = hdr_error_vs_f64(gpu_hdr, fr)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def visible_triangles(r, st, view):
    """Triangles of the view's visible meshlets: the draw commands' vertex
    counts / 3 (DrawIndirectCommand{3 * triangles, 1, 0, slot})."""
    import numpy as np
    o = r.out
    base = o.draw_calls + view * o.draw_call_section_bytes
    total = 0
    classes = ((0, min(st.visible_opaque[view], o.max_draws)),
               (o.max_draws, min(st.visible_alpha_clip[view], o.max_draws)))
    for first, n in classes:
        if n:
            cmds = r.download(base + 8 + 16 * first, 16 * n, np.uint32).reshape(n, 4)
            total += int(cmds[:, 0].astype(np.int64).sum()) // 3
    return total


def bench_batched(lh, torch, args, device):
    """Batched views (main 1920x1080 + 32 probes 64^2-512^2 + 4 cascades at
    2048^2, scene of the large configuration): device time per frame of the
    cull + raster + resolve under each launch schedule, CUDA-graph replayed."""
    scene = lh.Scene(3, seed=args.seed).upload(device)
    d = scene.desc
    probes, n = scene.probe_uniforms()
    px = 0
    for p in range(n):
        w, h = lh.uniforms_fields(probes[p])["window_size"]
        px += (w * h + 31) // 32 * 32
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=max(1024, d.n_instances),
                    max_draws=2000000, max_probes=n, max_probe_pixels=px, device=device)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    u = scene.uniforms
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = {"workload": "main %dx%d + %d probes (%d px) + 4 cascades %d^2" % (d.width, d.height, n, px, d.shadow_size)}
    out["autotuned"] = _autotune(r, u, stream, args, probes, n, frames=2)
    out["tuning"] = r.tuning().as_dict()
    for name, sched, graph in (("persistent_graph", lh.SCHEDULE_PERSISTENT, True),
                               ("per_stage_graph", lh.SCHEDULE_PER_STAGE, True),
                               ("per_stage_launches", lh.SCHEDULE_PER_STAGE, False),
                               ("per_view_graph", lh.SCHEDULE_PER_VIEW, True),
                               ("per_view_launches", lh.SCHEDULE_PER_VIEW, False)):
        r.set_tuning(schedule=sched)
        run = (lambda: r.frame_graph(u, probes, n, stream=sptr)) if graph else \
            (lambda: r.frame_batched(u, probes, n, stream=sptr))
        for _ in range(max(3, args.warmup)):
            run()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                ev[i][0].record(stream)
            run()
            with torch.cuda.stream(stream):
                ev[i][1].record(stream)
        torch.cuda.synchronize()
        out[name + "_ms"] = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    # where a batched frame's time goes (per-stage schedule, CUDA events)
    r.set_tuning(schedule=lh.SCHEDULE_PER_STAGE)
    r.set_profiling(True)
    r.frame_batched(u, probes, n, stream=sptr)
    out["per_stage_stage_ms"] = {k: round(v, 4) for k, v in r.stage_times().items()}
    r.set_profiling(False)
    st = r.status()
    out["status_flags"] = int(st.flags)
    out["visible_meshlets_all_views"] = int(sum(st.visible_opaque[v] for v in range(5 + n)))
    out["speedup_persistent_vs_per_view_launches"] = out["per_view_launches_ms"] / out["persistent_graph_ms"]
    best = min(("persistent_graph", "per_stage_graph", "per_stage_launches"), key=lambda k: out[k + "_ms"])
    out["best_batched"] = best
    out["speedup_best_batched_vs_per_view_launches"] = out["per_view_launches_ms"] / out[best + "_ms"]
    out["speedup_persistent_vs_per_view_graph"] = out["per_view_graph_ms"] / out["persistent_graph_ms"]
    return out


def bench_differentiable(lh, torch, args, device):
    """Differentiable resolve (2,048 instances of 4 meshes at 512x512): the
    forward resolve kernel and the adjoint (lh_resolve_backward with every
    gradient target) timed with CUDA events on one stream."""
    import ctypes as C
    import numpy as np
    from lighthugger_gb300.diff import _scene_records
    scene = lh.Scene(4, seed=args.seed).upload(device)
    d = scene.desc
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size,
                              max_instances=max(1024, d.n_instances), max_draws=2000000, device=device))
    r.set_scene(scene)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    u = scene.uniforms
    recs, inst = _scene_records(scene)
    dev = torch.device("cuda", device)
    total_v = sum(m.vertices for m in recs)
    g_pos = torch.zeros(total_v * 3, device=dev)
    g_nrm = torch.zeros(total_v * 3, device=dev)
    g_uv = torch.zeros(total_v * 2, device=dev)
    g_bcf = torch.zeros(len(recs) * 4, device=dev)
    first, rows = 0, []
    for k, m in enumerate(recs):
        rows.append([g_pos.data_ptr() + 12 * first, g_nrm.data_ptr() + 12 * first, g_uv.data_ptr() + 8 * first,
                     g_bcf.data_ptr() + 16 * k])
        first += m.vertices
    rec_dev = torch.tensor(np.array(rows, np.uint64).view(np.int64), device=dev)
    inst_rec = torch.tensor((rec_dev.data_ptr() + 32 * inst.astype(np.int64)), device=dev)
    tex_grads = [torch.zeros(t.width * t.height * 4, device=dev) for t in
                 (scene.desc.host_textures[i] for i in range(d.n_textures))]
    tex_tab = torch.tensor([t.data_ptr() for t in tex_grads], dtype=torch.int64, device=dev)
    light = torch.zeros(8, device=dev)
    grad = torch.randn(d.height, d.width, 4, device=dev)
    t = lh.GradTargets(instance_grads=inst_rec.data_ptr(), texture_grads=tex_tab.data_ptr(),
                       light_dir=light.data_ptr(), light_color=light.data_ptr() + 16)
    tuned = None
    if args.tune:
        # the adjoint's tile rows picked by the autotuner (before timing)
        from lighthugger_gb300 import autotune
        r.frame(u, stream=sptr)
        rows, res = autotune.tune_backward(r, grad.data_ptr(), t, frames=4, stream=stream)
        tuned = {"backward_rows": rows, "ms": {str(k): round(v, 4) for k, v in res.items()}}
    r.set_profiling(True)
    fwd, bwd = [], []
    for i in range(max(3, args.warmup) + args.steps):
        r.frame(u, stream=sptr)
        st_ms = r.stage_times()["resolve"]
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
        lh._check(lh.lib().lh_resolve_backward(r.ctx, grad.data_ptr(), C.byref(t), C.c_void_p(sptr)),
                  "lh_resolve_backward", r.ctx)
        with torch.cuda.stream(stream):
            b.record(stream)
        torch.cuda.synchronize()
        if i >= max(3, args.warmup):
            fwd.append(st_ms)
            bwd.append(a.elapsed_time(b))
    r.set_profiling(False)
    f_ms, b_ms = sum(fwd) / len(fwd), sum(bwd) / len(bwd)
    return {"workload": "%d instances of %d meshes, %dx%d, visibility fixed" % (d.n_instances, d.n_meshes, d.width,
                                                                                 d.height),
            "resolve_forward_ms": f_ms, "resolve_backward_ms": b_ms, "bwd_over_fwd": b_ms / f_ms,
            "backward_rows": int(r.tuning().backward_rows), "autotuned": tuned}


def bench_stress(lh, torch, args, device):
    """Stress workload (100,000 instances of 16 meshes up to 500k triangles,
    ~40M candidate meshlets, 3840x2160 + 4 cascades at 1024^2): the frame
    replayed from its CUDA graph, its stages, and the frame with the resolve
    adjoint captured in the same graph (lh_frame_graph_backward); CUDA events
    on one stream, L2 flushed between steps."""
    import ctypes as C
    import numpy as np
    from lighthugger_gb300.diff import _scene_records
    scene = lh.Scene(5, seed=args.seed).upload(device)
    d = scene.desc
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=d.n_instances,
                              max_draws=6000000, max_big_triangles=1 << 22, device=device))
    r.set_scene(scene)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    u = scene.uniforms
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    autotuned = _autotune(r, u, stream, args, frames=2)
    dev = torch.device("cuda", device)
    recs, inst = _scene_records(scene)
    total_v = sum(m.vertices for m in recs)
    g_pos, g_nrm = torch.zeros(total_v * 3, device=dev), torch.zeros(total_v * 3, device=dev)
    g_uv, g_bcf = torch.zeros(total_v * 2, device=dev), torch.zeros(len(recs) * 4, device=dev)
    rows, first = [], 0
    for k, m in enumerate(recs):
        rows.append([g_pos.data_ptr() + 12 * first, g_nrm.data_ptr() + 12 * first, g_uv.data_ptr() + 8 * first,
                     g_bcf.data_ptr() + 16 * k])
        first += m.vertices
    rec_dev = torch.tensor(np.array(rows, np.uint64).view(np.int64), device=dev)
    inst_rec = torch.tensor(rec_dev.data_ptr() + 32 * inst.astype(np.int64), device=dev)
    tex_grads = [torch.zeros(d.host_textures[i].width * d.host_textures[i].height * 4, device=dev)
                 for i in range(d.n_textures)]
    tex_tab = torch.tensor([t.data_ptr() for t in tex_grads], dtype=torch.int64, device=dev)
    light = torch.zeros(8, device=dev)
    grad = torch.randn(d.height, d.width, 4, device=dev, generator=torch.Generator(device=dev).manual_seed(3))
    t = lh.GradTargets(instance_grads=inst_rec.data_ptr(), texture_grads=tex_tab.data_ptr(),
                       light_dir=light.data_ptr(), light_color=light.data_ptr() + 16)

    def timed(run, steps):
        for _ in range(max(3, args.warmup)):
            run()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                ev[i][0].record(stream)
            run()
            with torch.cuda.stream(stream):
                ev[i][1].record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / steps

    steps = max(3, min(args.steps, 10))
    frame_ms = timed(lambda: r.frame_graph(u, None, 0, stream=sptr), steps)
    both_ms = timed(lambda: r.frame_graph_backward(u, None, 0, grad.data_ptr(), t, stream=sptr), steps)
    r.set_profiling(True)
    r.frame(u, stream=sptr)
    stage_ms = r.stage_times()
    r.set_profiling(False)
    st = r.status()
    out = {"workload": "%d instances of %d meshes, %.1fM triangles before culling, %dx%d + 4 cascades %d^2" % (
        d.n_instances, d.n_meshes, d.total_triangles / 1e6, d.width, d.height, d.shadow_size),
        "frame_graph_ms": frame_ms, "frame_and_backward_graph_ms": both_ms,
        "backward_ms": both_ms - frame_ms,
        "stage_ms": {k: round(v, 4) for k, v in stage_ms.items()},
        "candidate_meshlets": int(st.candidate_meshlets[0]), "visible_instances": int(st.visible_instances[0]),
        "visible_meshlets": int(st.visible_opaque[0] + st.visible_alpha_clip[0]),
        "shadow_candidate_meshlets": int(sum(st.candidate_meshlets[1:5])),
        "fragments": int(st.fragments[0]), "shadow_fragments": int(st.fragments[1]),
        "fragments_per_s": st.fragments[0] / (stage_ms["raster"] * 1e-3) if stage_ms["raster"] else None,
        # prefix-sum scale: candidate meshlets looked up per second by the meshlet cull
        "meshlet_cull_candidates_per_s": st.candidate_meshlets[0] / (stage_ms["cull_meshlets"] * 1e-3)
        if stage_ms["cull_meshlets"] else None,
        "occlusion": {"occluders": int(st.occlusion[0]), "survivors_opaque": int(st.occlusion[1]),
                      "survivors_alpha": int(st.occlusion[2])},
        "tuning": dict(r.tuning().as_dict(), autotuned=autotuned),
        "status_flags": int(st.flags), "steps": steps}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--cpu-frames", type=int, default=3)
    ap.add_argument("--batched", type=int, default=1, help="also time the batched multi-view frame (config 3)")
    ap.add_argument("--differentiable", type=int, default=1, help="also time the resolve adjoint (config 4)")
    ap.add_argument("--stress", type=int, default=1, help="also time the stress workload (config 5)")
    ap.add_argument("--tune", type=int, default=1, help="autotune the launch shape of each workload before timing it")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
