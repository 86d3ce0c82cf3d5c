"""Scene dumps (lh_scene_save / lh_scene_load, include/lh/scene.h): a scene
written to a file and read back gives the oracle the same frame as the
original (the golden digests of tests/golden/oracle_frames.json) and the
same description, probes included; incomplete or inconsistent files are
refused with a status, never read past."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from tests.conftest import ROOT

with open(os.path.join(ROOT, "tests", "golden", "oracle_frames.json")) as _f:
    _GOLDEN = json.load(_f)

DESC_FIELDS = ("config_id", "n_instances", "n_meshes", "n_textures", "n_probes", "width", "height", "shadow_size",
               "total_meshlets", "total_triangles", "seed")


@pytest.mark.parametrize("name", sorted(_GOLDEN))
def test_dump_replays_the_golden_frame(native, tmp_path, name):
    from tests.golden.make_golden import CASES, make_scene, scene_digest
    config_id, params = CASES[name]
    path = str(tmp_path / "scene.lhs")
    make_scene(config_id, params).save(path)
    loaded = native.Scene.load(path)
    got = scene_digest(loaded, config_id, params)
    want = _GOLDEN[name]
    for k in ("instances_sha256", "views", "visibility_sha256", "shadow_maps_sha256", "misc_sha256", "covered_pixels",
              "flags", "size", "shadow_size", "seed"):
        assert got[k] == want[k], "%s: %s differs" % (name, k)
    assert got["hdr_sum"] == pytest.approx(want["hdr_sum"], rel=1e-6)


def test_dump_keeps_the_description_and_probes(native, tmp_path):
    lh = native
    a = lh.Scene(3)
    path = str(tmp_path / "probes.lhs")
    a.save(path)
    b = lh.Scene.load(path)
    for k in DESC_FIELDS:
        assert getattr(a.desc, k) == getattr(b.desc, k), k
    assert bytes(a.uniforms) == bytes(b.uniforms)
    pa, n = a.probe_uniforms()
    pb, m = b.probe_uniforms()
    assert n == m == 32
    assert C.string_at(C.addressof(pa), n * lh.UNIFORMS_BYTES) == C.string_at(C.addressof(pb), n * lh.UNIFORMS_BYTES)
    # the same bytes when written again
    path2 = str(tmp_path / "again.lhs")
    b.save(path2)
    assert open(path, "rb").read() == open(path2, "rb").read()


def _expect_status(lh, path, status):
    with pytest.raises(lh.LHError) as e:
        lh.Scene.load(path)
    assert e.value.status == status


def test_broken_dumps_are_refused(native, tmp_path):
    lh = native
    path = str(tmp_path / "small.lhs")
    lh.Scene(1).save(path)
    raw = open(path, "rb").read()
    n = lh.Scene(1).desc.n_instances

    def variant(tag, data):
        p = str(tmp_path / (tag + ".lhs"))
        with open(p, "wb") as f:
            f.write(data)
        return p

    _expect_status(lh, str(tmp_path / "missing.lhs"), 7)                       # cannot be opened
    _expect_status(lh, variant("empty", b""), 1)
    _expect_status(lh, variant("magic", b"X" + raw[1:]), 1)
    _expect_status(lh, variant("version", raw[:8] + b"\x02\x00\x00\x00" + raw[12:]), 1)
    for cut in (len(raw) // 3, len(raw) // 2, len(raw) - 1):
        _expect_status(lh, variant("cut%d" % cut, raw[:cut]), 1)               # truncated
    _expect_status(lh, variant("tail", raw + b"\x00"), 1)                      # trailing bytes
    # the last instance's MeshInfo record index (the file's last 4 bytes) out of range
    _expect_status(lh, variant("record", raw[:-4] + b"\xff\xff\xff\xff"), 1)
    assert n > 0


def test_dump_of_a_caller_mesh(native, tmp_path):
    """lh_scene_from_mesh scenes (fp32 attributes, 32-bit indices) round trip
    to the same oracle frame."""
    lh = native
    from oracle import binding as ob
    small = lh.Scene(1)
    pos = np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3], [1, 3, 2]], np.uint32)
    tr = np.stack([np.eye(4, dtype=np.float32) for _ in range(3)])
    tr[:, 2, 3] = [-4.0, -6.0, -8.0]
    tr[:, 0, 3] = [0.0, 0.5, -0.5]
    a = lh.Scene.from_mesh(pos, idx, tr, small.uniforms)
    path = str(tmp_path / "mesh.lhs")
    a.save(path)
    b = lh.Scene.load(path)
    fa, fb = ob.run_scene(a, shadow_size=256), ob.run_scene(b, shadow_size=256)
    assert np.array_equal(fa.vis, fb.vis) and np.array_equal(fa.shadow, fb.shadow)
    assert np.array_equal(fa.misc, fb.misc)
