"""Edge-case geometry through the whole frame, GPU against the oracle, on a
caller mesh (lh_scene_from_mesh): a finely tessellated grid (shared edges
everywhere), duplicated and coplanar triangles (depth ties: the larger
packed ID wins), zero-area triangles (repeated and collinear vertices),
slivers, a triangle far larger than the view (chunks, guard band) and, from
a second camera, triangles through the near plane."""
import numpy as np
import pytest

from tests.parity import compare_frame

pytestmark = pytest.mark.gpu


def _edge_mesh():
    rng = np.random.default_rng(7)
    pos, tris = [], []

    def add(p):
        pos.append(p)
        return len(pos) - 1

    # 48 x 48 grid of quads on z = 0 over [-1, 1]^2, normals towards -z
    n = 48
    base = len(pos)
    for j in range(n + 1):
        for i in range(n + 1):
            add((-1.0 + 2.0 * i / n, -1.0 + 2.0 * j / n, 0.0))
    for j in range(n):
        for i in range(n):
            a = base + j * (n + 1) + i
            b, c, d = a + 1, a + n + 1, a + n + 2
            tris += [(a, c, b), (b, c, d)]
    # the same triangles again (ties at equal depth) and a coplanar
    # overlapping fan rotated by a few degrees
    tris += tris[: 2 * n]
    centre = add((0.1, 0.05, 0.0))
    ring = [add((0.1 + 0.6 * np.cos(t), 0.05 + 0.6 * np.sin(t), 0.0)) for t in np.linspace(0, 2 * np.pi, 97)[:-1]]
    for k in range(len(ring)):
        tris.append((centre, ring[(k + 1) % len(ring)], ring[k]))
    # zero-area triangles: a repeated vertex, collinear vertices
    p, q = add((0.3, 0.3, -0.01)), add((0.5, 0.32, -0.01))
    r_ = add((0.7, 0.34, -0.01))
    tris += [(p, p, q), (p, q, r_)]
    # slivers (aspect ~ 1000) in front of the grid
    for k in range(64):
        x, y = rng.uniform(-0.9, 0.9, 2)
        a = add((x, y, -0.02))
        b = add((x + 0.8, y + 0.0008, -0.02))
        c = add((x + 0.4, y + 0.0016, -0.02))
        tris.append((a, c, b))
    # a triangle far larger than the view, behind the grid
    tris.append((add((-60.0, -60.0, 0.5)), add((0.0, 80.0, 0.5)), add((60.0, -60.0, 0.5))))
    # tiny triangles, well below a pixel
    for k in range(256):
        x, y = rng.uniform(-0.95, 0.95, 2)
        a = add((x, y, -0.03))
        tris.append((a, add((x, y + 1e-4, -0.03)), add((x + 1e-4, y, -0.03))))
    return np.array(pos, np.float32), np.array(tris, np.uint32)


def _transforms():
    t0 = np.eye(4)
    t1 = np.eye(4)  # the same mesh again, a little behind and rotated about z
    c, s = np.cos(0.3), np.sin(0.3)
    t1[:2, :2] = [[c, -s], [s, c]]
    t1[2, 3] = 0.2
    t2 = np.eye(4)  # and exactly coplanar with the first, shifted by a third of a cell
    t2[0, 3] = 2.0 / 48 / 3
    return [t0, t1, t2]


@pytest.mark.parametrize("camera", ["front", "near"])
def test_edge_geometry_parity(native, oracle, camera):
    lh = native
    pos, tris = _edge_mesh()
    w, h = 640, 480
    if camera == "front":
        u = lh.make_uniforms((0.0, 0.0, -2.4), 1.5707963, 0.0, 60.0, w, h, 3)
    else:  # close enough that the grid crosses the near plane at the view's edge
        u = lh.make_uniforms((0.05, -0.1, -0.012), 1.5707963, 0.35, 100.0, w, h, 3)
    scene = lh.Scene.from_mesh(pos, tris, _transforms(), u).upload(0)
    d = scene.desc
    cfg = lh.Config(width=w, height=h, shadow_size=1024, max_instances=16, max_draws=200000)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    r.frame(scene.uniforms)
    st = r.status()
    fr = oracle.run_scene(scene, shadow_size=1024, max_instances=16, max_draws=200000)
    errors, stats = compare_frame(r, fr, 200000, 16)
    assert not errors, "\n".join(errors) + " %s" % stats
    assert st.flags == fr.flags
    assert stats["covered"] > 0.2 * w * h
    if camera == "near":
        assert fr.raster_stats["visibility"]["clipped"] > 0


_ORACLE_FRAMES = {}


@pytest.mark.parametrize("camera", ["front", "near"])
@pytest.mark.parametrize("shape", [(4, 32, 32, 256), (32, 256, 8, 64), (16, 128, 32, 32)])
def test_edge_geometry_all_triangles_in_chunks(native, oracle, camera, shape):
    """Every triangle with a pixel in its box through the big-triangle chunks
    (lane and warp bins off), at chunk shapes from 4 x 32 to 32 x 256 pixels:
    the chunks' runs of covered pixels give the oracle's visibility buffer
    and shadow maps bit for bit (slivers, ties, sub-pixel and clipped
    triangles included)."""
    lh = native
    pos, tris = _edge_mesh()
    w, h = 640, 480
    if camera == "front":
        u = lh.make_uniforms((0.0, 0.0, -2.4), 1.5707963, 0.0, 60.0, w, h, 3)
    else:
        u = lh.make_uniforms((0.05, -0.1, -0.012), 1.5707963, 0.35, 100.0, w, h, 3)
    scene = lh.Scene.from_mesh(pos, tris, _transforms(), u).upload(0)
    r = lh.Renderer(lh.Config(width=w, height=h, shadow_size=1024, max_instances=16, max_draws=200000))
    r.set_scene(scene)
    r.set_tuning(small_px=0, medium_px=0, chunk_rows=[shape[0], shape[2]], chunk_cols=[shape[1], shape[3]])
    r.frame(scene.uniforms)
    st = r.status()
    assert st.flags == 0, hex(st.flags)
    assert st.big_triangles > 1000
    if camera not in _ORACLE_FRAMES:
        _ORACLE_FRAMES[camera] = oracle.run_scene(scene, shadow_size=1024, max_instances=16, max_draws=200000)
    fr = _ORACLE_FRAMES[camera]
    errors, stats = compare_frame(r, fr, 200000, 16)
    assert not errors, "\n".join(errors) + " %s" % stats
