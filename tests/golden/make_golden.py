"""Writes tests/golden/oracle_frames.json: digests of the oracle's frame
outputs on four seeded scenes (the small scene, its quantized vertex
formats, the clustered large-scene layout at reduced detail, and the same
with alpha-clip materials).

The oracle cannot be checked against the reference's own outputs (the
reference is a Vulkan renderer with no CPU path, tests or vectors), so these
fixtures pin the oracle against itself: tests/test_golden.py recomputes each
frame and compares, so that an unintended change of the oracle or of the
scene generator shows up as a failing test.  Integer, visibility, depth and
shadow outputs are pinned by SHA-256 of their bytes; the HDR radiance by its
sum and largest value (float64, compared to a relative 1e-6).  Run from the
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


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def frame_digest(config_id, params):
    import ctypes as C

    import lighthugger_gb300 as lh
    from oracle import binding as ob
    scene = lh.Scene(config_id, **params)
    d = scene.desc
    fr = ob.run_scene(scene)
    # the Instance records with each mesh_info_address (bytes 64..71, a host
    # address that differs from run to run) replaced by its mesh's ordinal
    instances = np.frombuffer(C.string_at(d.host_instances, d.n_instances * lh.INSTANCE_BYTES), np.uint8)
    instances = instances.reshape(d.n_instances, lh.INSTANCE_BYTES).copy()
    addr = instances[:, 64:72].copy().view(np.uint64).ravel()
    ordinal = {a: i for i, a in enumerate(dict.fromkeys(addr.tolist()))}
    instances[:, 64:72] = np.array([ordinal[a] for a in addr.tolist()], np.uint64).view(np.uint8).reshape(-1, 8)
    covered = int(((fr.vis >> np.uint64(32)) != 0).sum())
    counts = []
    for v in range(5):
        sec = fr.sector(v)
        dr = fr.draw_section(v)
        counts.append({"instances": int(sec[:8].view(np.uint32)[1]),
                       "opaque": int(dr[:8].view(np.uint32)[0]), "alpha_clip": int(dr[:8].view(np.uint32)[1])})
    return {
        "config": config_id, "params": params, "seed": scene.seed,
        "size": [int(d.width), int(d.height)], "shadow_size": int(d.shadow_size),
        "instances_sha256": sha(instances),
        "counts": counts, "covered_pixels": covered, "flags": fr.flags,
        "prefix_sha256": sha(fr.prefix), "references_sha256": sha(fr.refs), "draws_sha256": sha(fr.draws),
        "visibility_sha256": sha(fr.vis), "shadow_maps_sha256": sha(fr.shadow), "misc_sha256": sha(fr.misc),
        "hdr_sum": float(fr.hdr.astype(np.float64).sum()), "hdr_max": float(fr.hdr.max()),
    }


def main():
    out = {name: frame_digest(cid, params) for name, (cid, params) in CASES.items()}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
