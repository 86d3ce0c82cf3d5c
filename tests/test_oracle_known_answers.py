"""Known-answer tests that pin the CPU oracle.

The reference has no tests, golden vectors or CPU path (it is a Vulkan
renderer that cannot run here), so the oracle is pinned by answers derived by
hand from the rules it restates: pixel-centre coverage with the top-left
rule, Vulkan's face orientation, clipping, the depth test, the packed
prefix-sum counter, the draw-command layout and the depth-range reduction.
"""
import numpy as np
import pytest

from tests import scene_view as sv


def clip_from_pixels(pts, W, H, z=0.5, w=1.0):
    """Clip-space vertices whose viewport position is `pts` (pixels)."""
    out = []
    for x, y in pts:
        out.append([(x / W * 2 - 1) * w, (y / H * 2 - 1) * w, z * w, w])
    return np.array(out, np.float32)


def covered(t):
    return (t >> np.uint64(32)) != 0


def test_right_triangle_pixel_count(oracle):
    # front facing (counter-clockwise in Vulkan's y-down sense): (0,0),(0,8),(8,0)
    t = oracle.raster_triangle(clip_from_pixels([(0, 0), (0, 8), (8, 0)], 8, 8), 77, 0, 8, 8)
    cov = covered(t)
    # centres with x + y <= 6 are inside; x + y = 7 lies on the hypotenuse, which is
    # not a top or left edge, so it is excluded
    ys, xs = np.mgrid[0:8, 0:8]
    assert np.array_equal(cov, xs + ys <= 6)
    assert cov.sum() == 28
    assert (t[cov] & np.uint64(0xFFFFFFFF) == 77).all()
    depth = (t[cov] >> np.uint64(32)).astype(np.uint32).view(np.float32)
    assert (depth == np.float32(0.5)).all()


def test_back_faces_culled_for_visibility_kept_for_shadows(oracle):
    ccw = clip_from_pixels([(0, 0), (0, 8), (8, 0)], 8, 8)
    cw = ccw[[0, 2, 1]]
    assert covered(oracle.raster_triangle(cw, 1, 0, 8, 8)).sum() == 0
    assert covered(oracle.raster_triangle(ccw, 1, 0, 8, 8)).sum() == 28
    # shadow kind keeps the min depth bits, culls front faces
    sh = oracle.raster_triangle(cw, 0, 1, 8, 8)
    assert ((sh & np.uint64(0xFFFFFFFF)) != 0x3F800000).sum() == 28
    sh2 = oracle.raster_triangle(ccw, 0, 1, 8, 8)
    assert ((sh2 & np.uint64(0xFFFFFFFF)) != 0x3F800000).sum() == 0


@pytest.mark.parametrize("diag", ["main", "anti"])
def test_shared_edge_watertight(oracle, diag):
    """Two triangles sharing the square's diagonal, which runs through pixel
    centres: every pixel is covered exactly once (top-left rule)."""
    W = H = 16
    if diag == "main":
        a = [(0, 0), (16, 16), (16, 0)]
        b = [(0, 0), (0, 16), (16, 16)]
    else:
        a = [(16, 0), (0, 0), (0, 16)]
        b = [(16, 0), (0, 16), (16, 16)]
    n = np.zeros((H, W), int)
    for tri in (a, b):
        for order in ([0, 1, 2], [0, 2, 1]):  # exactly one winding is front facing
            n += covered(oracle.raster_triangle(clip_from_pixels(tri, W, H)[order], 5, 0, W, H))
    assert (n == 1).all(), n


def test_depth_test_keeps_nearest_and_larger_id_on_ties(oracle):
    W = H = 8
    tri = clip_from_pixels([(0, 0), (0, 8), (8, 0)], W, H, z=0.25)
    near = clip_from_pixels([(0, 0), (0, 8), (8, 0)], W, H, z=0.75)  # reverse-Z: larger depth is nearer
    t = oracle.raster_triangle(tri, 3, 0, W, H)
    t = oracle.raster_triangle(near, 2, 0, W, H, t)
    cov = covered(t)
    assert (t[cov] & np.uint64(0xFFFFFFFF) == 2).all()
    t = oracle.raster_triangle(near, 9, 0, W, H, t)  # equal depth: larger packed ID wins
    assert (t[cov] & np.uint64(0xFFFFFFFF) == 9).all()


def test_near_plane_and_guard_band_clipping(oracle):
    """A triangle with a vertex behind the eye (z > w) and one far outside the
    guard band: clipped in clip space, the visible part covers the viewport."""
    W = H = 8
    near = 0.01
    # reverse-Z infinite projection: z_clip = near, w = distance
    verts = np.array([[-30, -30, near, 1.0], [30, -30, near, 1.0], [0, 4000, near, -0.5]], np.float32)
    cnt = 0
    for order in ([0, 1, 2], [0, 2, 1]):
        t = oracle.raster_triangle(verts[order], 4, 0, W, H)
        c = covered(t)
        cnt += c.sum()
        if c.any():
            d = (t[c] >> np.uint64(32)).astype(np.uint32).view(np.float32)
            assert ((d > 0) & (d <= 1)).all()
    assert cnt > 0
    # entirely behind the near plane: nothing
    behind = np.array([[-1, -1, near, -1.0], [1, -1, near, -1.0], [0, 1, near, -1.0]], np.float32)
    for order in ([0, 1, 2], [0, 2, 1]):
        assert covered(oracle.raster_triangle(behind[order], 4, 0, W, H)).sum() == 0


def test_subpixel_triangle_between_centres(oracle):
    tri = clip_from_pixels([(1.1, 1.1), (1.1, 1.4), (1.4, 1.1)], 8, 8)
    for order in ([0, 1, 2], [0, 2, 1]):
        assert covered(oracle.raster_triangle(tri[order], 1, 0, 8, 8)).sum() == 0


def test_prefix_sector_and_draw_lists_structure(native, oracle):
    """Canonical order and the packed {count:hi32, sum:lo32} counter."""
    lh = native
    scene = lh.Scene(1)
    fr = oracle.run_scene(scene, shadow_size=256, max_instances=1024, max_draws=200000)
    sec = fr.sector(0)
    counter = int(sec[:8].view(np.uint64)[0])
    count, total = counter >> 32, counter & 0xFFFFFFFF
    vals = sec[8:8 + 8 * count].view(np.uint32).reshape(-1, 2)
    inst = sv.instances(scene)
    nm = np.array([int(sv.mesh_info(int(a))["num_meshlets"]) for a in inst["mesh_info_address"]])
    assert (np.diff(vals[:, 0].astype(np.int64)) > 0).all()
    assert np.array_equal(vals[:, 1], np.cumsum(nm[vals[:, 0]]))
    assert total == vals[-1, 1]
    ds = fr.draw_section(0)
    nop = int(ds[:4].view(np.uint32)[0])
    dc = ds[8:8 + 16 * nop].view(np.uint32).reshape(-1, 4)
    refs = fr.meshlet_references(0)[:8 * nop].view(np.uint32).reshape(-1, 2)
    assert np.array_equal(dc[:, 3], np.arange(nop))  # firstInstance = slot
    assert (dc[:, 1] == 1).all() and (dc[:, 2] == 0).all()
    key = refs[:, 0].astype(np.int64) * 65536 + (refs[:, 1] & 0xFFFF)
    assert (np.diff(key) > 0).all()  # instance ascending, then meshlet ascending
    for k in range(0, nop, max(1, nop // 50)):
        mi = sv.mesh_info(int(inst["mesh_info_address"][refs[k, 0]]))
        ml = sv.read(int(mi["meshlets"]) + 56 * int(refs[k, 1] & 0xFFFF), 56).view(sv.MESHLET_DTYPE)[0]
        assert dc[k, 0] == 3 * int(ml["triangle_count"])


def test_depth_range_reduction(native, oracle):
    """read_depth.glsl: min over non-zero depth bits, max over all."""
    scene = native.Scene(1)
    fr = oracle.run_scene(scene, shadow_size=256)
    d = (fr.vis >> np.uint64(32)).astype(np.uint32)
    m = fr.misc[784:792].view(np.uint32)
    assert m[0] == d[d != 0].min() and m[1] == d.max()
    radii = fr.misc[768:784].view(np.float32)
    assert (radii > 0).all() and np.array_equal(radii * 16, np.round(radii * 16))


def test_resolve_float_vs_float64(native, oracle):
    """The oracle's float resolve against its float64 twin: the HDR error of
    the reference's float math itself, bounded at its 99th percentile over
    covered pixels."""
    scene = native.Scene(1, width=320, height=180)
    fr = oracle.run_scene(scene, shadow_size=512)
    h64 = oracle.resolve_f64(fr)
    cov = covered(fr.vis)
    err = np.abs(fr.hdr[..., :3].astype(np.float64) - h64[..., :3])
    # kink pixels (shadow compare / cascade choice flipping) aside, float32 is ~1e-6 relative
    assert np.percentile(err[cov], 99) < 1e-4


def _alpha_texture():
    """2 x 1 RGBA8 texture: texel 0 alpha 0, texel 1 alpha 255."""
    t = np.zeros((1, 2, 4), np.uint8)
    t[0, 1, 3] = 255
    return t


def test_alpha_clip_keeps_fragments_where_alpha_reaches_half(oracle):
    # u = x / 16 across a 16 x 16 target; the bilinear, repeat-addressed alpha
    # of the 2-texel texture is >= 0.5 exactly for u in [0.5, 1], so only the
    # right half's pixel centres (x >= 8) survive
    W = H = 16
    clip = clip_from_pixels([(0, 0), (0, 32), (32, 0)], W, H)
    uv = np.array([[0, 0.5], [0, 0.5], [2, 0.5]], np.float32)
    t = oracle.raster_triangle_alpha(clip, uv, _alpha_texture(), 2, 1, 9, 0, W, H)
    ys, xs = np.mgrid[0:H, 0:W]
    assert np.array_equal(covered(t), xs >= 8)
    # double sided: the other winding covers the same fragments (an opaque
    # draw of it is culled)
    t2 = oracle.raster_triangle_alpha(clip[[0, 2, 1]], uv[[0, 2, 1]], _alpha_texture(), 2, 1, 9, 0, W, H)
    assert np.array_equal(covered(t2), xs >= 8)
    assert covered(oracle.raster_triangle(clip[[0, 2, 1]], 9, 0, W, H)).sum() == 0


def test_alpha_clip_uv_is_perspective_correct(oracle):
    # same screen triangle with w = 1, 2, 4 at its vertices: the surviving
    # pixels follow the perspective-correct u, computed here in float64
    W = H = 16
    pts = [(0, 0), (0, 32), (32, 0)]
    ws = [1.0, 2.0, 4.0]
    clip = np.concatenate([clip_from_pixels([p], W, H, w=w) for p, w in zip(pts, ws)])
    u = np.array([0.0, 0.0, 2.0])
    uv = np.stack([u, np.full(3, 0.5)], 1).astype(np.float32)
    t = oracle.raster_triangle_alpha(clip, uv, _alpha_texture(), 2, 1, 3, 0, W, H)
    ys, xs = np.mgrid[0:H, 0:W].astype(np.float64)
    X, Y = (xs + 0.5), (ys + 0.5)
    # screen-space barycentrics of the pixel centre, then perspective correction
    b2 = X / 32.0
    b1 = Y / 32.0
    b0 = 1.0 - b1 - b2
    q = np.stack([b0 / ws[0], b1 / ws[1], b2 / ws[2]])
    lam = q / q.sum(0)
    uu = (lam * u[:, None, None]).sum(0)
    ut = uu * 2 - 0.5
    a = ut - np.floor(ut)
    i0 = np.floor(ut).astype(int) % 2
    alpha = np.where(i0 == 0, a, 1 - a)  # texel 0 has alpha 0, texel 1 alpha 1
    clear = np.abs(alpha - 0.5) > 1e-3
    assert clear.sum() > 200
    assert np.array_equal(covered(t)[clear], (alpha >= 0.5)[clear])


def test_display_transform_known_values(oracle):
    # identity stand-in LUT: display = stimulus / (1 + stimulus), then the
    # sRGB transfer function and rounding to 8 bits
    stim = np.array([0.0, 1.0, 3.0, 1e-4], np.float32)
    hdr = np.zeros((1, 4, 4), np.float32)
    hdr[0, :, 0] = hdr[0, :, 1] = hdr[0, :, 2] = stim
    out = oracle.display_transform(hdr)
    enc = stim.astype(np.float64) / (stim + 1.0)
    srgb = np.where(enc <= 0.00313, enc * 12.92, 1.055 * enc ** (1 / 2.4) - 0.055)
    expect = np.floor(np.clip(srgb, 0, 1) * 255 + 0.5)
    assert np.array_equal(out[0, :, 0], expect.astype(np.uint8)), (out[0, :, 0], expect)
    assert (out[..., 3] == 255).all()
    # a full LUT of one colour maps everything to it
    lut = np.zeros((48, 48, 48, 4), np.float32)
    lut[..., 1] = 0.5
    out = oracle.display_transform(hdr, lut=lut)
    assert (out[0, :, 0] == 0).all() and (out[0, :, 1] == 188).all()


def test_display_transform_shadow_overlay(oracle):
    # debug_shadowmaps: the top-left quarter shows the 4 cascades at
    # (depth - 0.5) * 100 + 0.5; a map of 0.5 reads back as 0.5 -> 188
    W = H = 16
    hdr = np.zeros((H, W, 4), np.float32)
    maps = np.full((4, 8, 8), 0.5, np.float32)
    maps[3] = 0.51  # cascade 3 (bottom-right of the quarter): 1.5 -> white
    out = oracle.display_transform(hdr, shadow_maps=maps, debug_shadowmaps=1)
    assert (out[:4, :4, 0] == 188).all()
    assert (out[4:8, 4:8, 0] == 255).all()
    assert (out[8:, :, 0] == 0).all() and (out[:, 8:, 0] == 0).all()
