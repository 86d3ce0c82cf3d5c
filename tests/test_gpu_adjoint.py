"""Resolve adjoint on the GPU (lh_resolve_backward) against the oracle's FP64
reference gradient: central differences (h = 1e-4) of the FP64 forward
resolve over the same float buffers, visibility held fixed, upstream
gradient N(0,1) on interior pixels (>= 2 px inside their triangle) and zero
elsewhere.  Workload: the differentiable-resolve configuration at its full
size (2,048 instances of 4 meshes, 512 x 512).  Parameters: vertex positions,
normals and uvs of triangles under those pixels, per-material base-colour
factors, light direction and colour, and texels -- base-colour texels and the
metallic-roughness texel whose green channel is the roughness and blue the
metalness (render_geometry.comp:233-236).

Error bound 1e-3 on the relative error of each kind's vector of checked
gradients, ||g_gpu - g_fp64|| / ||g_fp64||.  Each component is also checked,
at 1e-2 relative to the larger of its own size and 5% of the kind's largest,
to catch a gross error in one entry: single components are sums that nearly
cancel (the upstream gradient has random signs), so float32 rounding of the
per-pixel terms is amplified in them -- a uv gradient adds terms of size
texture width x texel difference (~10 here), and the float32 sample position
(u x width, ~1e-4 texel of rounding) moves the other axis' bilinear weight
by as much; a material's roughness gradient sums ~700 pixels' BRDF terms of
both signs.  Measured: components of 0.8 and 0.38 off by 2e-3 and 1.2e-3
relative while every kind's vector stays within 1e-3."""
COMPONENT_TOL = 1e-2
import ctypes as C

import numpy as np
import pytest

from tests import scene_view as sv

pytestmark = pytest.mark.gpu

REL_TOL = 1e-3


def _interior_pixels(vis, margin=2):
    ids = (vis & np.uint64(0xFFFFFFFF)).astype(np.int64)
    cov = (vis >> np.uint64(32)) != 0
    ok = cov.copy()
    H, W = vis.shape
    for dy in range(-margin, margin + 1):
        for dx in range(-margin, margin + 1):
            sh = np.full_like(ids, -1)
            ys = slice(max(dy, 0), H + min(dy, 0))
            yd = slice(max(-dy, 0), H + min(-dy, 0))
            xs = slice(max(dx, 0), W + min(dx, 0))
            xd = slice(max(-dx, 0), W + min(-dx, 0))
            sh[yd, xd] = ids[ys, xs]
            ok &= sh == ids
    return ok


class HostScene:
    """Writable views of the host scene's float buffers (what the oracle reads)."""

    def __init__(self, scene):
        self.scene = scene
        self.inst = sv.instances(scene)
        self.infos = {}
        for a in self.inst["mesh_info_address"]:
            a = int(a)
            if a not in self.infos:
                self.infos[a] = sv.Mesh(sv.mesh_info(a))

    def float_view(self, addr, n):
        return np.ctypeslib.as_array((C.c_float * n).from_address(addr))

    def vertex_arrays(self, info_addr):
        m = self.infos[info_addr]
        nv = len(m.positions)
        mi = m.mi
        return (self.float_view(int(mi["positions"]), nv * 3).reshape(nv, 3),
                self.float_view(int(mi["normals"]), nv * 3).reshape(nv, 3),
                self.float_view(int(mi["uvs"]), nv * 2).reshape(nv, 2))

    def bcf_view(self, info_addr):
        return self.float_view(info_addr + 92, 3)


def _smooth_pixels(oracle, fr, hs, textures, trials=4, h=2e-4):
    """Pixels whose FP64 radiance responds smoothly to joint random
    perturbations of every parameter (no clamp, texel centre, face sign,
    cascade or shadow-compare switch within reach): the second difference
    must stay far below the first.  The reach (2e-4, relative) is twice the
    central differences' step, so no kink lies inside their window."""
    rng = np.random.default_rng(3)
    arrays = []
    for a in hs.infos:
        arrays += list(hs.vertex_arrays(a)) + [hs.bcf_view(a)]
    arrays.append(np.ctypeslib.as_array((C.c_float * 140).from_address(C.addressof(fr._ubuf)))[127:133])
    arrays += list(textures)
    base = oracle.resolve_f64(fr)[..., :3]
    ok = np.ones(base.shape[:2], bool)
    for _ in range(trials):
        saved = [x.copy() for x in arrays]
        dirs = [rng.choice([-1.0, 1.0], size=x.shape) * np.maximum(1.0, np.abs(x)) * h for x in saved]
        res = []
        for sgn in (1.0, -1.0):
            for x, x0, dx in zip(arrays, saved, dirs):
                x[...] = (x0 + sgn * dx).astype(np.float32)
            res.append(oracle.resolve_f64(fr)[..., :3])
        for x, x0 in zip(arrays, saved):
            x[...] = x0
        first = np.abs(res[0] - res[1]).sum(-1)
        second = np.abs(res[0] + res[1] - 2 * base).sum(-1)
        ok &= second <= 0.02 * first + 1e-12
    return ok


def _texture_linear(r, n_textures):
    """The context's linear float4 copies of the textures (what the kernels
    sample), as float32 [h, w, 4] host arrays."""
    out = []
    for i in range(n_textures):
        addr, w, h = r.texture_linear(i)
        out.append(r.download(addr, w * h * 16, np.float32).reshape(h, w, 4).copy())
    return out


def _adjoint_checks(lh, oracle, scene, r, u):
    """GPU adjoint of the frame seen with uniforms `u` against FP64 central
    differences: returns the (kind, gpu, fp64, where) checks and the skipped
    count."""
    import torch
    d = scene.desc
    r.frame(u)
    fr = oracle.run_scene(scene, shadow_size=d.shadow_size, max_instances=max(1024, d.n_instances),
                          max_draws=400000, uniforms=u)
    vis = fr.vis
    assert np.array_equal(r.visibility(), vis)
    hs = HostScene(scene)
    # the FP64 resolve samples the very texels the kernels sample (float32
    # values; its own RGBA8 decode divides in float64): the image moves by
    # rounding only
    tex = _texture_linear(r, d.n_textures)
    before = oracle.resolve_f64(fr)
    tex = oracle.set_linear_textures(fr, tex)
    base = oracle.resolve_f64(fr)
    assert float(np.nanmax(np.abs(base - before))) < 1e-6
    interior = _interior_pixels(vis) & _smooth_pixels(oracle, fr, hs, tex)
    # pixels the sun reaches (the sun term changes with the light colour):
    # roughness and metalness act there through the BRDF, so the picks are
    # drawn from them (in shadow only the ambient term is left)
    ub = np.ctypeslib.as_array((C.c_float * 140).from_address(C.addressof(fr._ubuf)))
    saved = ub[130:133].copy()
    ub[130:133] = 0.0
    dark = oracle.resolve_f64(fr)
    ub[130:133] = saved
    lit = np.abs(base - dark)[..., :3].sum(-1) > 1e-3 * np.abs(base)[..., :3].sum(-1) + 1e-9
    interior &= lit
    rng = np.random.default_rng(11)
    ys, xs = np.nonzero(interior)
    assert len(ys) > 400, "too few interior pixels: %d" % len(ys)
    pick = rng.choice(len(ys), size=min(800, len(ys)), replace=False)
    G = np.zeros((d.height, d.width, 4), np.float32)
    G[ys[pick], xs[pick], :3] = rng.normal(size=(len(pick), 3)).astype(np.float32)
    xy = np.stack([xs[pick], ys[pick]], axis=1)
    Gp = G[ys[pick], xs[pick], :3].astype(np.float64)

    # ---- GPU adjoint into per-vertex-buffer, per-record and per-texture
    # buffers: MeshInfo records of one mesh with different materials share
    # its vertex buffers, so their vertex gradients go to one buffer (what a
    # central difference of a shared vertex sees)
    info_addrs = sorted(hs.infos)
    dev = torch.device("cuda")
    vbufs, bufs = {}, {}
    rec = np.zeros((len(info_addrs), 4), np.uint64)
    for k, a in enumerate(info_addrs):
        nv = len(hs.infos[a].positions)
        key = int(hs.infos[a].mi["positions"])
        if key not in vbufs:
            vbufs[key] = {"pos": torch.zeros(nv * 3, device=dev), "nrm": torch.zeros(nv * 3, device=dev),
                          "uv": torch.zeros(nv * 2, device=dev)}
        b = dict(vbufs[key])
        b["bcf"] = torch.zeros(4, device=dev)
        bufs[a] = b
        rec[k] = [b["pos"].data_ptr(), b["nrm"].data_ptr(), b["uv"].data_ptr(), b["bcf"].data_ptr()]
    rec_dev = torch.from_numpy(rec.view(np.int64)).to(dev)
    inst_rec = np.array([rec_dev.data_ptr() + 32 * info_addrs.index(int(a)) for a in hs.inst["mesh_info_address"]],
                        np.uint64)
    inst_rec_dev = torch.from_numpy(inst_rec.view(np.int64)).to(dev)
    tex_grads = [torch.zeros(t.size, device=dev) for t in tex]
    tex_tab = torch.tensor([t.data_ptr() for t in tex_grads], dtype=torch.int64, device=dev)
    light = torch.zeros(8, device=dev)
    g_dev = torch.from_numpy(G).to(dev)
    t = lh.GradTargets(instance_grads=inst_rec_dev.data_ptr(), texture_grads=tex_tab.data_ptr(),
                       light_dir=light.data_ptr(), light_color=light.data_ptr() + 16)
    torch.cuda.synchronize()
    st = lh.lib().lh_resolve_backward(r.ctx, g_dev.data_ptr(), C.byref(t), None)
    assert st == 0
    torch.cuda.synchronize()
    gpu = {a: {k: v.cpu().numpy().astype(np.float64) for k, v in b.items()} for a, b in bufs.items()}
    gl = light.cpu().numpy().astype(np.float64)
    gtex = [g.cpu().numpy().astype(np.float64).reshape(tx.shape) for g, tx in zip(tex_grads, tex)]

    # ---- FP64 reference: L(theta) = sum G . hdr64 over the picked pixels
    def loss():
        return float((oracle.resolve_f64_pixels(fr, xy)[:, :3] * Gp).sum())

    def fd(arr, i, h):
        """Central difference of L in arr[i] (a float32 view) with exact steps."""
        x0 = arr[i]

        def at(step):
            arr[i] = np.float32(x0 + step)
            dx = float(arr[i]) - float(x0)
            v = loss()
            arr[i] = x0
            return v, dx

        (lp, dp), (lm, dm) = at(h), at(-h)
        (lp2, dp2), (lm2, dm2) = at(h / 2), at(-h / 2)
        g1 = (lp - lm) / (dp - dm)
        g2 = (lp2 - lm2) / (dp2 - dm2)
        return g1, abs(g1 - g2) <= 1e-3 * (abs(g1) + abs(g2)) + 1e-9

    checks, skipped = [], 0

    def record(kind, got, ref, ok, where=""):
        nonlocal skipped
        if not ok:
            skipped += 1
            return
        checks.append((kind, got, ref, where))

    # vertices of triangles under picked pixels
    vis_p = vis[ys[pick], xs[pick]]
    slots = (vis_p & np.uint64(0xFFFFFF)).astype(np.int64)
    tris = (vis_p >> np.uint64(24) & np.uint64(0xFF)).astype(np.int64)
    refs = fr.meshlet_references(0).view(np.uint32).reshape(-1, 2)
    verts = []
    for s_, t_ in list(zip(slots, tris))[:12]:
        inst_i = int(refs[s_, 0])
        ml_i = int(refs[s_, 1] & 0xFFFF)
        a = int(hs.inst["mesh_info_address"][inst_i])
        micro, idx = hs.infos[a].meshlet_triangles(ml_i)
        verts.append((a, int(idx[t_][0])))
    verts = list(dict.fromkeys(verts))[:8]
    for a, vi in verts:
        P, N, UV = hs.vertex_arrays(a)
        for c in range(3):
            g, ok = fd(P[vi], c, 1e-4 * max(1.0, abs(float(P[vi][c]))))
            record("position", gpu[a]["pos"][vi * 3 + c], g, ok, "mesh %#x vertex %d axis %d" % (a, vi, c))
            g, ok = fd(N[vi], c, 1e-4)
            record("normal", gpu[a]["nrm"][vi * 3 + c], g, ok, "mesh %#x vertex %d axis %d" % (a, vi, c))
        for c in range(2):
            g, ok = fd(UV[vi], c, 1e-4)
            record("uv", gpu[a]["uv"][vi * 2 + c], g, ok, "mesh %#x vertex %d axis %d" % (a, vi, c))
    for a in info_addrs[:3]:
        bv = hs.bcf_view(a)
        for c in range(3):
            g, ok = fd(bv, c, 1e-4)
            record("base_color_factor", gpu[a]["bcf"][c], g, ok)
    for c in range(3):
        g, ok = fd(ub, 127 + c, 1e-4)  # sun_dir at byte 508
        record("light_dir", gl[c], g, ok)
        g, ok = fd(ub, 130 + c, 1e-4)  # sun_intensity at byte 520
        record("light_color", gl[4 + c], g, ok)
    # texels: per texture the few with the largest GPU gradient.  1 x 1
    # textures are the metallic-roughness ones (green = roughness, blue =
    # metalness); the 256 x 256 ones the base colours (rgb)
    kinds = {"roughness": 0, "metalness": 0, "base_color_texel": 0}
    for i, (tx, gt) in enumerate(zip(tex, gtex)):
        h_, w_ = tx.shape[:2]
        flat = tx.reshape(-1)
        gflat = gt.reshape(-1)
        if h_ * w_ == 1:
            for ch, kind in ((1, "roughness"), (2, "metalness")):
                if gflat[ch] == 0.0 or kinds[kind] >= 8:
                    continue  # material not under a picked pixel / enough checks
                g, ok = fd(flat, ch, 1e-4)
                record(kind, gflat[ch], g, ok)
                kinds[kind] += 1
        elif kinds["base_color_texel"] < 24:
            rgb = np.abs(gt[..., :3]).reshape(-1)
            for k in np.argsort(rgb)[::-1][:4]:
                if rgb[k] == 0.0:
                    break
                j = (k // 3) * 4 + k % 3
                g, ok = fd(flat, j, 1e-4)
                record("base_color_texel", gflat[j], g, ok)
                kinds["base_color_texel"] += 1

    return checks, skipped


def test_adjoint_matches_fp64_central_differences(native, oracle):
    """The differentiable-resolve workload at full size, seen from its own
    camera and from one 4 m higher looking 0.3 rad down (from the first, the
    lit interior pixels are nearly all on two materials; the second adds
    three more)."""
    lh = native
    scene = lh.Scene(4).upload(0)
    d = scene.desc
    assert (d.n_instances, d.width, d.height) == (2048, 512, 512)
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size,
                              max_instances=max(1024, d.n_instances), max_draws=400000))
    r.set_scene(scene)
    cam = lh.uniforms_fields(scene.uniforms)["camera_pos"].astype(float)
    high = lh.make_uniforms((cam[0], cam[1] + 4.0, cam[2]), 1.0, -0.3, 60.0, d.width, d.height, d.n_instances)
    checks, skipped, worst = [], 0, 0.0
    for cam_i, u in enumerate((scene.uniforms, high)):
        c, sk = _adjoint_checks(lh, oracle, scene, r, u)
        checks += [(k, g, f, "camera %d %s" % (cam_i, w)) for k, g, f, w in c]
        skipped += sk
    assert len(checks) >= 120, "only %d checks (%d skipped)" % (len(checks), skipped)
    by_kind = {}
    for kind, got, ref, where in checks:
        by_kind.setdefault(kind, []).append((got, ref, where))
    need = {"roughness": 4, "metalness": 4, "base_color_texel": 8, "position": 8, "normal": 8, "uv": 8,
            "base_color_factor": 4, "light_dir": 2, "light_color": 2}
    for kind, n in need.items():
        assert len(by_kind.get(kind, [])) >= n, "too few %s checks: %s" % (kind, {k: len(v) for k, v in by_kind.items()})
    report, vec_err = [], {}
    for kind, lst in by_kind.items():
        gots = np.array([a for a, b, w in lst])
        refs_ = np.array([b for a, b, w in lst])
        scale = max(np.abs(refs_).max(), 1e-6)
        vec_err[kind] = float(np.linalg.norm(gots - refs_) / max(np.linalg.norm(refs_), 1e-12))
        if vec_err[kind] > REL_TOL:
            report.append("%s: vector relative error %.2e" % (kind, vec_err[kind]))
        for got, ref, where in lst:
            err = abs(got - ref) / max(abs(ref), 5e-2 * scale)
            worst = max(worst, err)
            if err > COMPONENT_TOL:
                report.append("%s %s: gpu %.8g fp64 %.8g rel %.2e" % (kind, where, got, ref, err))
    assert not report, "\n".join(report[:20]) + "\n(%d checks, %d skipped)" % (len(checks), skipped)
    print("adjoint: %d checks (%s), %d skipped, worst component error %.2e, vector errors %s" % (
        len(checks), {k: len(v) for k, v in by_kind.items()}, skipped, worst,
        {k: "%.1e" % v for k, v in vec_err.items()}))
