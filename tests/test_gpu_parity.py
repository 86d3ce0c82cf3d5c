"""CUDA path (through the C ABI) against the CPU oracle on seeded scenes.

Bit exact: prefix-sum sectors, visible-meshlet lists, draw commands,
visibility IDs and depth, MiscStorage (cascade fit), shadow maps.
Within 2^-10 max abs: linear HDR radiance.
"""
import numpy as np
import pytest

from tests.parity import compare_frame

pytestmark = pytest.mark.gpu


def _run(native, oracle, config_id, seed=None, max_draws=200000, max_instances=None, frames=1, **params):
    lh = native
    scene = lh.Scene(config_id, seed=seed, **params).upload(0)
    d = scene.desc
    cap = max_instances or max(1024, d.n_instances)
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=cap,
                    max_draws=max_draws, device=0)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    for _ in range(frames):
        r.frame(scene.uniforms)
    st = r.status()
    fr = oracle.run_scene(scene, shadow_size=d.shadow_size, max_instances=cap, max_draws=max_draws)
    return scene, r, fr, st, cap


def _assert_parity(r, fr, md, cap, st, fr_flags=None):
    errors, stats = compare_frame(r, fr, md, cap)
    assert not errors, "\n".join(errors) + "\nstats %s" % stats
    if fr_flags is not None:
        assert st.flags == fr_flags, "device flags %#x oracle %#x" % (st.flags, fr_flags)
    return stats


def test_config1_frame_parity(native, oracle):
    scene, r, fr, st, cap = _run(native, oracle, 1)
    stats = _assert_parity(r, fr, 200000, cap, st, fr.flags)
    assert stats["covered"] > 1000
    assert st.visible_opaque[0] > 0


def test_config1_repeat_frames_identical(native, oracle):
    """Two frames in a row give identical results (counters reset, canonical order)."""
    scene, r, fr, st, cap = _run(native, oracle, 1, frames=2)
    _assert_parity(r, fr, 200000, cap, st)


def test_config1_quantized_formats(native, oracle):
    """Reference vertex formats: u16 positions, i8 normals, u16 uvs, 16-bit indices."""
    scene, r, fr, st, cap = _run(native, oracle, 1, quantized=1)
    _assert_parity(r, fr, 200000, cap, st)


def test_config1_reference_normal_transform(native, oracle):
    """normal_transform = mat3(inverse(M)) exactly as the reference's Instance constructor."""
    scene, r, fr, st, cap = _run(native, oracle, 1, reference_normal_transform=1)
    _assert_parity(r, fr, 200000, cap, st)


def test_config2_reduced_parity(native, oracle):
    """Config 2 layout (clustered scene, textured materials) at reduced mesh detail."""
    scene, r, fr, st, cap = _run(native, oracle, 2, detail=0.25, n_instances=1024, width=960, height=540)
    stats = _assert_parity(r, fr, 200000, cap, st)
    assert stats["covered"] > 10000


def test_config1_alpha_clip_double_sided(native, oracle):
    """Alpha-clip materials with opaque constant textures: every alpha-class
    meshlet is rasterised double sided and passes the alpha test."""
    scene, r, fr, st, cap = _run(native, oracle, 1, alpha_clip_materials=1)
    stats = _assert_parity(r, fr, 200000, cap, st, fr.flags)
    assert st.visible_alpha_clip[0] > 0
    assert stats["covered"] > 1000


def test_config2_alpha_clip_parity(native, oracle):
    """Textured alpha-clip materials with holes: the per-fragment alpha test
    (bilinear alpha at the perspective-correct uv) discards bit-exactly as
    the oracle, in the visibility buffer and the shadow maps."""
    scene, r, fr, st, cap = _run(native, oracle, 2, detail=0.25, n_instances=1024, width=960, height=540,
                                 alpha_clip_materials=1)
    stats = _assert_parity(r, fr, 200000, cap, st)
    assert st.visible_alpha_clip[0] > 0 and stats["covered"] > 10000


def test_alpha_clip_scene_after_opaque_scene(native, oracle):
    """The alpha-class raster launches are left out for a scene without
    alpha-clip meshes; the same renderer given a scene with them (a second
    lh_set_scene) rasterises them again, through the per-stage launches and
    the replayed graph."""
    lh = native
    opaque = lh.Scene(1).upload(0)
    alpha = lh.Scene(1, alpha_clip_materials=1).upload(0)
    d = alpha.desc
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=1024,
                    max_draws=200000, device=0)
    r = lh.Renderer(cfg)
    r.set_scene(opaque)
    r.frame_graph(opaque.uniforms)
    assert r.status().visible_alpha_clip[0] == 0
    r.set_scene(alpha)
    fr = oracle.run_scene(alpha, shadow_size=d.shadow_size, max_instances=1024, max_draws=200000)
    for run in (lambda: r.frame(alpha.uniforms), lambda: r.frame_graph(alpha.uniforms)):
        run()
        st = r.status()
        assert st.visible_alpha_clip[0] > 0
        _assert_parity(r, fr, 200000, 1024, st, fr.flags)


def test_config2_full_parity(native, oracle):
    """Config 2 at full size: 4,096 instances, ~50M triangles, 1920x1080."""
    scene, r, fr, st, cap = _run(native, oracle, 2)
    stats = _assert_parity(r, fr, 200000, cap, st)
    assert stats["covered"] > 100000
    # without the occlusion test every visible meshlet is rasterised: the
    # raster's fragment counters (its depth-test reductions) then equal the
    # oracle's covered, alpha-passed fragments of the same frame
    r.set_tuning(occlusion_px=0)
    r.frame(scene.uniforms)
    st0 = r.status()
    _assert_parity(r, fr, 200000, cap, st0)
    rs = fr.raster_stats
    assert (st0.fragments[0], st0.fragments[1]) == (rs["visibility"]["fragments"], rs["shadow"]["fragments"])
    # with it, the skipped meshlets' fragments are never issued
    assert st.fragments[0] < st0.fragments[0] and st.fragments[1] == st0.fragments[1]


def test_occlusion_raster_is_exact(native, oracle):
    """The two-pass occlusion raster (occluders, hierarchical depth, depth
    test of every other meshlet's sphere, survivors) gives the same bits as
    the one-pass raster and the oracle, at several occluder thresholds, and
    at the large configuration it skips most meshlets."""
    lh = native
    scene = lh.Scene(2).upload(0)
    d = scene.desc
    cap = max(1024, d.n_instances)
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=cap,
                              max_draws=200000))
    r.set_scene(scene)
    u = scene.uniforms
    fr = oracle.run_scene(scene, shadow_size=d.shadow_size, max_instances=cap, max_draws=200000)
    outs = {}
    for px in (0, 4, 32, 128, 1024):
        r.set_tuning(occlusion_px=px)
        r.frame(u)
        st = r.status()
        assert st.flags == 0, (px, hex(st.flags))
        errors, stats = compare_frame(r, fr, 200000, cap)
        assert not errors, (px, errors)
        outs[px] = (r.visibility(), r.hdr(), r.shadow_maps(), st)
        if px:
            occ, surv_op, surv_al = (int(x) for x in st.occlusion)
            assert 0 < occ < st.visible_opaque[0]
            assert surv_op + occ <= st.visible_opaque[0] and surv_al <= st.visible_alpha_clip[0]
    for px in (4, 32, 128, 1024):
        assert np.array_equal(outs[px][0], outs[0][0]) and np.array_equal(outs[px][2], outs[0][2])
        assert np.array_equal(outs[px][1], outs[0][1])
    st = outs[128][3]
    # the near object hides most of the view: most meshlets never reach the raster
    assert st.occlusion[0] + st.occlusion[1] < 0.2 * st.visible_opaque[0], list(st.occlusion)


def test_overflow_capacities_flagged(native, oracle):
    """Capacities below need: work is dropped and flagged, never written out of bounds."""
    scene, r, fr, st, cap = _run(native, oracle, 1, max_draws=500, max_instances=16)
    assert st.flags & native.FLAG_INSTANCE_OVERFLOW
    assert st.flags & native.FLAG_DRAW_OVERFLOW
    assert fr.flags & native.FLAG_INSTANCE_OVERFLOW
    _assert_parity(r, fr, 500, 16, st)


def test_empty_view(native, oracle):
    """Camera looking away from everything: no visible instances, all-sky frame."""
    lh = native
    scene = lh.Scene(1).upload(0)
    d = scene.desc
    u = lh.make_uniforms((0.0, 0.0, -150.0), -1.5707963, 0.0, 60.0, d.width, d.height, d.n_instances)
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=1024, max_instances=1024, max_draws=200000)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    r.frame(u)
    st = r.status()
    fr = oracle.run_scene(scene, shadow_size=1024, max_instances=1024, max_draws=200000, uniforms=u)
    assert st.visible_instances[0] == 0
    assert st.flags & lh.FLAG_NO_DEPTH
    errors, _ = compare_frame(r, fr, 200000, 1024)
    assert not errors, errors


@pytest.mark.parametrize("schedule", ["per_stage", "per_view", "persistent"])
def test_zero_instances(native, schedule):
    """A frame with no instances after one with many: every target is cleared
    (visibility 0, shadow depth 1.0) although no instance is culled or drawn
    (the targets are cleared beside the instance cull, which then has no
    tiles)."""
    lh = native
    scene = lh.Scene(1).upload(0)
    d = scene.desc
    u = scene.uniforms
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=256, max_instances=1024, max_draws=100000)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    r.set_tuning(schedule={"per_stage": lh.SCHEDULE_PER_STAGE, "per_view": lh.SCHEDULE_PER_VIEW,
                           "persistent": lh.SCHEDULE_PERSISTENT}[schedule])
    r.frame(u)
    assert (r.visibility() != 0).any() and (r.shadow_maps() != 1.0).any()
    # uniforms.num_instances = 0: nothing is culled or drawn
    b = bytearray(bytes(u))
    b[532:536] = (0).to_bytes(4, "little")
    u0 = lh.Uniforms.from_buffer_copy(bytes(b))
    r.frame(u0)
    st = r.status()
    assert st.visible_instances[0] == 0 and st.visible_opaque[0] == 0
    assert (r.visibility() == 0).all()
    assert (r.shadow_maps() == 1.0).all()


def _camera_at_surface(lh, scene, inst_index, gap):
    """Uniforms for a camera `gap` metres above instance `inst_index`'s
    surface, looking along the surface: triangles under the eye reach from
    behind it to far in front, so they cross the near plane (gap < 0.01)
    and leave the guard band, and must be clipped."""
    from tests import scene_view as sv
    inst = sv.instances(scene)[inst_index]
    T = inst["transform"]  # [col][row]
    centre = T[3][:3].astype(np.float64)
    mi = sv.mesh_info(int(inst["mesh_info_address"]))
    bs = mi["bounding_sphere"].astype(np.float64)
    scale = max(np.linalg.norm(T[c][:3]) for c in range(3))
    centre = centre + sum(T[c][:3] * bs[c] for c in range(3))
    radius = bs[3] * scale
    n = np.array([0.3, 0.2, -1.0])
    n /= np.linalg.norm(n)
    eye = centre + n * (radius * 0.999 + gap)
    f = np.cross(n, [0.0, 1.0, 0.0])
    f /= np.linalg.norm(f)
    f = f - n * 0.05  # dip slightly towards the surface
    f /= np.linalg.norm(f)
    yaw, pitch = float(np.arctan2(f[2], f[0])), float(np.arcsin(f[1]))
    d = scene.desc
    return lh.make_uniforms(tuple(float(x) for x in eye), yaw, pitch, 60.0, d.width, d.height, d.n_instances)


@pytest.mark.parametrize("gap", [0.004, 0.5])
def test_near_plane_clipping_parity(native, oracle, gap):
    """Camera against an object's surface: near-plane and guard-band clipping."""
    lh = native
    scene = lh.Scene(1, width=640, height=360).upload(0)
    d = scene.desc
    u = _camera_at_surface(lh, scene, 3, gap)
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=512, max_instances=1024, max_draws=200000)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    r.frame(u)
    st = r.status()
    fr = oracle.run_scene(scene, shadow_size=512, max_instances=1024, max_draws=200000, uniforms=u)
    errors, stats = compare_frame(r, fr, 200000, 1024)
    assert not errors, "\n".join(errors) + " %s" % stats
    assert stats["covered"] > 0.05 * d.width * d.height  # the surface fills part of the view
    if gap < 0.01:
        assert fr.raster_stats["visibility"]["clipped"] > 0


@pytest.mark.parametrize("mode", [1, 2, 3, 5])
def test_debug_views(native, oracle, mode):
    """Uniforms.debug (render_geometry.comp:268-308): cascades, triangle
    index, meshlet index and normal colours match the oracle."""
    import ctypes
    lh = native
    scene = lh.Scene(1).upload(0)
    d = scene.desc
    u = lh.Uniforms.from_buffer_copy(bytes(scene.uniforms))
    ctypes.memmove(ctypes.addressof(u) + 552, ctypes.byref(ctypes.c_int32(mode)), 4)
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=1024, max_draws=200000)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    r.frame(u)
    st = r.status()
    fr = oracle.run_scene(scene, shadow_size=d.shadow_size, max_instances=1024, max_draws=200000, uniforms=u)
    _assert_parity(r, fr, 200000, 1024, st)
    hdr = r.hdr()
    lit = oracle.run_scene(scene, shadow_size=d.shadow_size, max_instances=1024, max_draws=200000)
    covered = (r.visibility() >> np.uint64(32)) != 0
    assert not np.array_equal(hdr[covered], lit.hdr[covered])  # the view replaced the lighting


@pytest.mark.parametrize("shadow_size,width,height", [(2048, 1280, 720), (1000, 1001, 601)])
def test_shadow_sizes_and_odd_widths(native, oracle, shadow_size, width, height):
    """Cascades whose PCF taps are not one texel apart (2048: two texels,
    1000: 0.98) take the per-tap path; an odd width (rows of the visibility
    buffer not 16-byte aligned) takes the resolve without TMA staging."""
    lh = native
    scene = lh.Scene(1, width=width, height=height).upload(0)
    d = scene.desc
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=shadow_size, max_instances=1024, max_draws=200000)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    r.frame(scene.uniforms)
    st = r.status()
    fr = oracle.run_scene(scene, shadow_size=shadow_size, max_instances=1024, max_draws=200000)
    errors, stats = compare_frame(r, fr, 200000, 1024)
    assert not errors, "\n".join(errors) + " %s" % stats
    assert st.flags == fr.flags
    assert stats["covered"] > 1000


def test_hdr_rgba16f_is_the_rgba32f_image_rounded(native):
    """LH_CONFIG_HDR_RGBA16F: every channel is the RGBA32F result rounded to
    nearest-even half (numpy's float16 conversion), alpha 1; the pipelined
    readback copies 8 bytes per pixel."""
    import torch
    lh = native
    scene = lh.Scene(1).upload(0)
    d = scene.desc
    out = {}
    for flags in (0, lh.CONFIG_HDR_RGBA16F):
        cfg = lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=1024,
                        max_draws=200000, flags=flags)
        r = lh.Renderer(cfg)
        r.set_scene(scene)
        r.frame(scene.uniforms)
        out[flags] = r.hdr().copy()
        if flags:
            buf = torch.empty(d.width * d.height * 4, dtype=torch.float16, pin_memory=True)
            r.frame_readback(scene.uniforms, buf.data_ptr())
            r.readback_wait()
            out["readback"] = buf.numpy().reshape(d.height, d.width, 4).copy()
    h16 = out[lh.CONFIG_HDR_RGBA16F]
    assert h16.dtype == np.float16
    assert np.array_equal(h16.view(np.uint16), out[0].astype(np.float16).view(np.uint16))
    assert np.all(h16[..., 3] == 1.0)
    assert np.array_equal(out["readback"].view(np.uint16), h16.view(np.uint16))

