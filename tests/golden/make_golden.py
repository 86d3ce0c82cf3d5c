"""Writes tests/golden/oracle_frames.json: digests of the oracle's frame
outputs on four seeded scenes (the small scene, its quantized vertex
formats, the clustered large-scene layout at reduced detail, and the same
with alpha-clip materials).

The oracle cannot be checked against the reference's own outputs (the
reference is a Vulkan renderer with no CPU path, tests or vectors), so these
fixtures pin the oracle against itself: tests/test_golden.py recomputes each
frame and compares, so that an unintended change of the oracle or of the
scene generator shows up as a failing test, and tests/test_gpu_golden.py
holds the CUDA path's frames of the same scenes to the same digests.
Integer, visibility, depth and shadow outputs are pinned by SHA-256 of their
bytes in a form both sides give; the HDR radiance by its sum and largest
value (float64).  Run from the
repository root after an intended change:

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

CASES = {
    "small": (1, {}),
    "small_quantized": (1, {"quantized": 1}),
    "clustered_reduced": (2, {"detail": 0.25, "n_instances": 1024, "width": 960, "height": 540}),
    "clustered_reduced_alpha_clip": (2, {"detail": 0.25, "n_instances": 1024, "width": 960, "height": 540,
                                         "alpha_clip_materials": 1}),
}
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_frames.json")


MAX_DRAWS = 200000


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def canonical_digest(sector, draw_section, references, vis, shadow, misc, hdr, md, cap):
    """Digests of a frame's outputs in the form both the oracle and the CUDA
    path give them: per view the prefix counter and entries up to the count,
    the draw counts, the listed draw commands and meshlet references (their
    padding bytes masked); visibility, shadow maps and MiscStorage (NaN
    words made one NaN) as bytes; the HDR sum and maximum."""
    from tests.parity import draw_lists, sector_entries
    views = []
    for v in range(5):
        counter, entries = sector_entries(sector(v), cap)
        (nop, nal), dc, rf = draw_lists(draw_section(v), references(v), md)
        views.append({"counter": counter, "opaque": nop, "alpha_clip": nal, "entries_sha256": sha(entries),
                      "draws_sha256": sha(dc), "references_sha256": sha(rf)})
    m = np.array(misc, dtype=np.uint8).view(np.uint32).copy()
    m[np.isnan(m.view(np.float32))] = 0x7FC00000
    return {"views": views, "covered_pixels": int(((vis >> np.uint64(32)) != 0).sum()),
            "visibility_sha256": sha(vis), "shadow_maps_sha256": sha(np.asarray(shadow).view(np.uint32)),
            "misc_sha256": sha(m), "hdr_sum": float(np.asarray(hdr, np.float64).sum()), "hdr_max": float(hdr.max())}


def make_scene(config_id, params):
    import lighthugger_gb300 as lh
    return lh.Scene(config_id, **params)


def instances_digest(scene):
    """The Instance records with each mesh_info_address (bytes 64..71, an
    address that differs from run to run) replaced by its mesh's ordinal."""
    import ctypes as C

    import lighthugger_gb300 as lh
    d = scene.desc
    raw = np.frombuffer(C.string_at(d.host_instances, d.n_instances * lh.INSTANCE_BYTES), np.uint8)
    inst = raw.reshape(d.n_instances, lh.INSTANCE_BYTES).copy()
    addr = inst[:, 64:72].copy().view(np.uint64).ravel()
    ordinal = {a: i for i, a in enumerate(dict.fromkeys(addr.tolist()))}
    inst[:, 64:72] = np.array([ordinal[a] for a in addr.tolist()], np.uint64).view(np.uint8).reshape(-1, 8)
    return sha(inst)


def frame_digest(config_id, params):
    """The oracle's frame of the config's scene, digested."""
    return scene_digest(make_scene(config_id, params), config_id, params)


def scene_digest(scene, config_id, params):
    """The oracle's frame of `scene`, digested."""
    from oracle import binding as ob
    d = scene.desc
    cap = max(1024, d.n_instances)
    fr = ob.run_scene(scene, max_instances=cap, max_draws=MAX_DRAWS)
    out = canonical_digest(fr.sector, fr.draw_section, fr.meshlet_references, fr.vis, fr.shadow, fr.misc, fr.hdr,
                           MAX_DRAWS, cap)
    out.update({"config": config_id, "params": params, "seed": scene.seed, "size": [int(d.width), int(d.height)],
                "shadow_size": int(d.shadow_size), "instances_sha256": instances_digest(scene), "flags": fr.flags})
    return out


def main():
    out = {name: frame_digest(cid, params) for name, (cid, params) in CASES.items()}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
