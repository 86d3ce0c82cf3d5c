"""Stress configuration: 100,000 instances of 16 meshes (up to 500k
triangles, long thin slivers included), 40.3M meshlets before culling,
3840x2160 + 4 cascades, depth complexity ~30 -- bit-exact against the oracle,
plain and batched (persistent) schedules."""
import ctypes

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


_REDUCED = {}


@pytest.mark.parametrize("occlusion_px", [128, 16])
def test_stress_reduced_parity(native, oracle, occlusion_px):
    """The stress scene's meshes at a quarter of its instances, 1920 x 1080
    + 4 cascades: bit exact against the oracle (a stress-shaped case small
    enough for a full profiler capture), with few occluders and with many
    (16 px: most tested meshlets are small and take the per-pixel test)."""
    lh = native
    scene = lh.Scene(5, n_instances=25000, width=1920, height=1080).upload(0)
    d = scene.desc
    md = 2000000
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=d.n_instances,
                              max_draws=md, max_big_triangles=1 << 21))
    r.set_scene(scene)
    r.set_tuning(occlusion_px=occlusion_px)
    r.frame(scene.uniforms)
    st = r.status()
    assert st.flags == 0, hex(st.flags)
    if "fr" not in _REDUCED:
        _REDUCED["fr"] = oracle.run_scene(scene, shadow_size=d.shadow_size, max_instances=d.n_instances, max_draws=md)
    errors, stats = compare_frame(r, _REDUCED["fr"], md, d.n_instances)
    assert not errors, "\n".join(errors) + " %s" % stats
    assert st.candidate_meshlets[0] > 1_000_000
    if occlusion_px == 16:
        assert st.occlusion[0] > 10_000 and st.occlusion[1] < st.visible_opaque[0] - st.occlusion[0]


def _grad_targets(lh, scene, torch):
    """Gradient buffers for every mesh record, texture and the light, and the
    GradTargets that point at them."""
    from lighthugger_gb300.diff import _scene_records
    recs, inst = _scene_records(scene)
    total_v = sum(m.vertices for m in recs)
    bufs = {"pos": torch.zeros(total_v * 3, device="cuda"), "nrm": torch.zeros(total_v * 3, device="cuda"),
            "uv": torch.zeros(total_v * 2, device="cuda"), "bcf": torch.zeros(len(recs) * 4, device="cuda"),
            "light": torch.zeros(8, device="cuda")}
    rows, first = [], 0
    for k, m in enumerate(recs):
        rows.append([bufs["pos"].data_ptr() + 12 * first, bufs["nrm"].data_ptr() + 12 * first,
                     bufs["uv"].data_ptr() + 8 * first, bufs["bcf"].data_ptr() + 16 * k])
        first += m.vertices
    bufs["rec"] = torch.tensor(np.array(rows, np.uint64).view(np.int64), device="cuda")
    bufs["inst"] = torch.tensor(bufs["rec"].data_ptr() + 32 * inst.astype(np.int64), device="cuda")
    d = scene.desc
    bufs["tex"] = [torch.zeros(d.host_textures[i].width * d.host_textures[i].height * 4, device="cuda")
                   for i in range(d.n_textures)]
    bufs["tex_tab"] = torch.tensor([t.data_ptr() for t in bufs["tex"]], dtype=torch.int64, device="cuda")
    t = lh.GradTargets(instance_grads=bufs["inst"].data_ptr(), texture_grads=bufs["tex_tab"].data_ptr(),
                       light_dir=bufs["light"].data_ptr(), light_color=bufs["light"].data_ptr() + 16)
    return t, bufs


def test_stress_frame_and_backward_in_one_graph(native, stress):
    """The batched forward and the resolve adjoint captured in one CUDA graph:
    the visibility equals the plain frame's and the gradients equal those of
    a separate lh_resolve_backward after it (up to the order of float atomics)."""
    import torch
    lh = native
    scene, r, _ = stress
    d = scene.desc
    grad = torch.randn(d.height, d.width, 4, device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    t1, b1 = _grad_targets(lh, scene, torch)
    t2, b2 = _grad_targets(lh, scene, torch)
    r.set_tuning(schedule=lh.SCHEDULE_PERSISTENT)
    r.frame_batched(scene.uniforms, None, 0)
    vis_plain = r.visibility().copy()
    torch.cuda.synchronize()
    lh._check(lh.lib().lh_resolve_backward(r.ctx, grad.data_ptr(), ctypes.byref(t1), r.stream), "backward", r.ctx)
    for _ in range(2):  # capture, then replay
        for b in (b2["pos"], b2["nrm"], b2["uv"], b2["bcf"], b2["light"], *b2["tex"]):
            b.zero_()
        torch.cuda.synchronize()
        r.frame_graph_backward(scene.uniforms, None, 0, grad.data_ptr(), t2)
        st = r.status()
        assert st.flags == 0, hex(st.flags)
        assert np.array_equal(r.visibility(), vis_plain)
        for key in ("pos", "nrm", "uv", "bcf", "light"):
            a, b = b1[key], b2[key]
            scale = float(a.abs().max()) + 1e-30
            assert float((a - b).abs().max()) <= 1e-4 * scale, key
        assert float(b2["pos"].abs().sum()) > 0
        ta = torch.cat(b1["tex"])
        tb = torch.cat(b2["tex"])
        assert float((ta - tb).abs().max()) <= 1e-4 * (float(ta.abs().max()) + 1e-30)
