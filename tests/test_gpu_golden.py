"""The CUDA path's frames of the golden scenes (tests/golden/
oracle_frames.json) against the committed digests: per view the prefix
sector, draw counts, draw commands and meshlet references, the visibility
buffer, shadow maps and MiscStorage bit for bit, the HDR sum to a relative
1e-5 and its maximum to 2^-10 -- the same fixtures the oracle is held to
(tests/test_golden.py), so both sides answer to the committed vectors as well
as to each other."""
import json
import os

import pytest

from tests.conftest import ROOT
from tests.golden.make_golden import CASES, MAX_DRAWS, canonical_digest, make_scene

pytestmark = pytest.mark.gpu

with open(os.path.join(ROOT, "tests", "golden", "oracle_frames.json")) as _f:
    _GOLDEN = json.load(_f)


@pytest.mark.parametrize("name", sorted(_GOLDEN))
def test_cuda_frame_matches_golden_digests(native, name):
    lh = native
    want = _GOLDEN[name]
    config_id, params = CASES[name]
    scene = make_scene(config_id, params).upload(0)
    d = scene.desc
    cap = max(1024, d.n_instances)
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=cap,
                              max_draws=MAX_DRAWS, device=0))
    r.set_scene(scene)
    r.frame(scene.uniforms)
    got = canonical_digest(r.prefix_sector, r.draw_section, r.meshlet_references, r.visibility(), r.shadow_maps(),
                           r.misc(), r.hdr(), MAX_DRAWS, cap)
    for k in ("views", "covered_pixels", "visibility_sha256", "shadow_maps_sha256", "misc_sha256"):
        assert got[k] == want[k], "%s: %s differs" % (name, k)
    assert r.status().flags == want["flags"]
    assert got["hdr_sum"] == pytest.approx(want["hdr_sum"], rel=1e-5)
    assert abs(got["hdr_max"] - want["hdr_max"]) <= 2.0 ** -10


def test_cuda_frame_from_a_scene_dump(native, tmp_path):
    """A golden scene written to a dump (lh_scene_save), read back
    (lh_scene_load) and uploaded renders the golden frame on the GPU."""
    lh = native
    name = "clustered_reduced_alpha_clip"
    want = _GOLDEN[name]
    config_id, params = CASES[name]
    path = str(tmp_path / "scene.lhs")
    make_scene(config_id, params).save(path)
    scene = lh.Scene.load(path).upload(0)
    d = scene.desc
    cap = max(1024, d.n_instances)
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=cap,
                              max_draws=MAX_DRAWS, device=0))
    r.set_scene(scene)
    r.frame(scene.uniforms)
    got = canonical_digest(r.prefix_sector, r.draw_section, r.meshlet_references, r.visibility(), r.shadow_maps(),
                           r.misc(), r.hdr(), MAX_DRAWS, cap)
    for k in ("views", "covered_pixels", "visibility_sha256", "shadow_maps_sha256", "misc_sha256"):
        assert got[k] == want[k], "%s: %s differs" % (name, k)
