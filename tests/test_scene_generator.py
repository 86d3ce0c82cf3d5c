"""Seeded scene generator: determinism and the invariants the pipeline relies on
(meshletiser limits of src/shared_cpu_gpu.h:148-150, 4-byte aligned triangle
offsets as at src/resources/meshlets.cpp:62-64, conservative normal cones
for the test of src/shaders/common/culling.glsl:137-151, bounding spheres)."""
import numpy as np
import pytest

from tests import scene_view as sv


def _meshes(scene):
    inst = sv.instances(scene)
    seen = {}
    for a in inst["mesh_info_address"]:
        a = int(a)
        if a not in seen:
            seen[a] = sv.Mesh(sv.mesh_info(a))
    return list(seen.values())


def test_deterministic(native):
    lh = native
    a, b = lh.Scene(1), lh.Scene(1)
    assert bytes(a.uniforms) == bytes(b.uniforms)
    assert np.array_equal(sv.instances(a)["transform"], sv.instances(b)["transform"])
    c = lh.Scene(1, seed=7)
    assert not np.array_equal(sv.instances(a)["transform"], sv.instances(c)["transform"])


@pytest.mark.parametrize("config,params", [(1, {}), (1, {"quantized": 1}), (2, {"detail": 0.1, "n_instances": 64}),
                                           (5, {"detail": 0.02, "n_instances": 200, "width": 256, "height": 144})])
def test_meshlet_invariants(native, config, params):
    scene = native.Scene(config, **params)
    for mesh in _meshes(scene):
        m = mesh.meshlets
        assert (m["index_count"] <= 64).all() and (m["index_count"] > 0).all()
        assert (m["triangle_count"] <= 124).all() and (m["triangle_count"] > 0).all()
        assert (m["triangle_offset"] % 4 == 0).all()
        for k in range(0, len(m), max(1, len(m) // 40)):
            micro, idx = mesh.meshlet_triangles(k)
            assert (micro < int(m[k]["index_count"])).all()
            pts = mesh.positions[idx.reshape(-1)]
            c = m[k]["bounding_sphere"][:3].astype(np.float64)
            r = float(m[k]["bounding_sphere"][3])
            assert (np.linalg.norm(pts - c, axis=1) <= r * (1 + 1e-5) + 1e-6).all()
        bs = mesh.mi["bounding_sphere"].astype(np.float64)
        assert (np.linalg.norm(mesh.positions - bs[:3], axis=1) <= bs[3] * (1 + 1e-5) + 1e-6).all()


def test_cones_are_conservative(native):
    """A viewpoint for which the cone test culls sees every triangle from behind."""
    scene = native.Scene(2, detail=0.1, n_instances=16)
    rng = np.random.default_rng(5)
    checked = 0
    for mesh in _meshes(scene):
        m = mesh.meshlets
        for k in range(0, len(m), max(1, len(m) // 25)):
            cut = float(m[k]["cone_cutoff"])
            if cut > 1:
                continue
            apex = m[k]["cone_apex"].astype(np.float64)
            axis = m[k]["cone_axis"].astype(np.float64)
            _, idx = mesh.meshlet_triangles(k)
            tri = mesh.positions[idx]
            n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
            r = float(m[k]["bounding_sphere"][3])
            for _ in range(40):
                d = rng.normal(size=3)
                d /= np.linalg.norm(d)
                eye = apex - d * rng.uniform(0.1, 50) * max(r, 1e-3)
                v = apex - eye
                if np.dot(v / np.linalg.norm(v), axis) >= cut:
                    # culled: every triangle must face away (dot(p - eye, n) >= 0)
                    assert (np.einsum("ij,ij->i", tri[:, 0] - eye, n) >= -1e-9 * np.abs(n).sum(1)).all()
                    checked += 1
    assert checked > 0


def test_uniforms_projection(native):
    """infinite_reverse_z_perspective (src/projection.h:3-20): y = -f, w = -z_view, z = near."""
    lh = native
    u = lh.make_uniforms((1.0, 2.0, 3.0), 0.3, -0.1, 60.0, 1920, 1080, 10)
    f = lh.uniforms_fields(u)
    P = f["perspective"]  # [col][row]
    fl = 1.0 / np.tan(np.radians(60.0) / 2)
    assert np.isclose(P[1][1], -fl, rtol=1e-6)
    assert np.isclose(P[0][0], fl / (1920 / 1080), rtol=1e-6)
    assert P[2][3] == -1.0 and np.isclose(P[3][2], 0.01)
    assert f["window_size"] == (1920, 1080) and f["num_instances"] == 10
    PV = f["combined_perspective_view"].T.astype(np.float64)
    inv = f["inv_perspective_view"].T.astype(np.float64)
    assert np.allclose(PV @ inv, np.eye(4), atol=1e-4)


def test_scene_from_mesh_builds_and_validates(native):
    """lh_scene_from_mesh: a caller mesh is meshletised (every triangle lands
    in one meshlet, <= 64 vertices and <= 124 triangles each) and bad input
    is refused."""
    lh = native
    rng = np.random.default_rng(3)
    pos = rng.uniform(-1, 1, (500, 3)).astype(np.float32)
    tris = rng.integers(0, 500, (700, 3)).astype(np.uint32)
    u = lh.make_uniforms((0.0, 0.0, -3.0), 1.5707963, 0.0, 60.0, 320, 200, 2)
    s = lh.Scene.from_mesh(pos, tris, [np.eye(4), np.eye(4)], u)
    d = s.desc
    assert (d.n_instances, d.n_meshes, d.width, d.height) == (2, 1, 320, 200)
    assert d.total_triangles == 2 * 700
    assert 700 / 124 <= d.total_meshlets / 2 <= 700
    bad = tris.copy()
    bad[5, 1] = 500  # index out of range
    with pytest.raises(lh.LHError):
        lh.Scene.from_mesh(pos, bad, [np.eye(4)], u)
    nan = pos.copy()
    nan[3, 0] = np.nan
    with pytest.raises(lh.LHError):
        lh.Scene.from_mesh(nan, tris, [np.eye(4)], u)
