"""Stress configuration: 100,000 instances of 16 meshes (up to 500k
triangles, long thin slivers included), 40.3M meshlets before culling,
3840x2160 + 4 cascades, depth complexity ~30 -- bit-exact against the oracle,
plain and batched (persistent) schedules."""
import numpy as np
import pytest

from tests.parity import compare_frame

pytestmark = pytest.mark.gpu

MAX_DRAWS = 6_000_000


@pytest.fixture(scope="module")
def stress(native, oracle):
    lh = native
    scene = lh.Scene(5).upload(0)
    d = scene.desc
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=d.n_instances,
                    max_draws=MAX_DRAWS, max_big_triangles=1 << 22)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    fr = oracle.run_scene(scene, shadow_size=d.shadow_size, max_instances=d.n_instances, max_draws=MAX_DRAWS)
    return scene, r, fr


@pytest.mark.parametrize("schedule", ["per_stage", "persistent"])
def test_stress_parity(native, stress, schedule):
    lh = native
    scene, r, fr = stress
    r.set_tuning(schedule=lh.SCHEDULE_PER_STAGE if schedule == "per_stage" else lh.SCHEDULE_PERSISTENT)
    r.frame_batched(scene.uniforms, None, 0)
    st = r.status()
    assert st.flags == 0, hex(st.flags)
    assert fr.flags == 0
    errors, stats = compare_frame(r, fr, MAX_DRAWS, scene.desc.n_instances)
    assert not errors, "\n".join(errors) + " %s" % stats
    assert stats["covered"] == scene.desc.width * scene.desc.height
    assert st.candidate_meshlets[0] > 5_000_000
