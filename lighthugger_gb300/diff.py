"""Differentiable lighting resolve for PyTorch.

`DiffResolve(renderer, scene)` exposes the scene's vertex positions, normals,
uvs and per-record base-colour factors as flat float32 CUDA tensors, the
linear RGBA texels of every texture (base colour; metallic-roughness, whose
green channel is the roughness and blue the metalness,
render_geometry.comp:233-236), plus the light direction and colour; calling
it renders one frame through the C ABI and returns the HDR image as a tensor
whose backward is the hand-written adjoint (lh_resolve_backward), wrapped in
a libtorch torch::autograd::Function
(lighthugger_gb300/torch_ext/diff_resolve.cpp).  Forward and backward run on
PyTorch's current CUDA stream.

Visibility is held fixed: the backward differentiates the lighting of the
forward's visibility buffer (triangle IDs, cascades and shadow-map compare
results are discrete and constant).
"""
import ctypes as C
import os

import numpy as np

from . import LIB_PATH, Uniforms, _check, lib, uniforms_fields

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
_ext = None


class SceneMesh(C.Structure):
    _fields_ = [("host_info", C.c_void_p), ("device_info", C.c_uint64), ("device_positions", C.c_uint64),
                ("device_normals", C.c_uint64), ("device_uvs", C.c_uint64), ("mesh", C.c_uint32),
                ("vertices", C.c_uint32), ("triangles", C.c_uint32), ("flags", C.c_uint32)]


def extension():
    """Build (in-tree, once) and load the libtorch extension."""
    global _ext
    if _ext is not None:
        return _ext
    from torch.utils.cpp_extension import load
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    build_dir = os.path.join(_HERE, "_build", "torch_ext")
    os.makedirs(build_dir, exist_ok=True)
    lib()  # the C ABI library must be there
    _ext = load(name="lh_torch_ext", sources=[os.path.join(_HERE, "torch_ext", "diff_resolve.cpp")], with_cuda=True,
                extra_include_paths=[os.path.join(_ROOT, "include"), os.path.join(cuda_home, "include")],
                extra_cflags=["-O2"],
                extra_ldflags=["-L" + os.path.dirname(LIB_PATH), "-l:liblh.so",
                               "-Wl,-rpath," + os.path.dirname(LIB_PATH), "-L" + os.path.join(cuda_home, "lib64"),
                               "-lcudart"],
                build_directory=build_dir, verbose=False)
    return _ext


def _scene_records(scene):
    L = lib()
    L.lh_scene_mesh_count.argtypes = [C.c_void_p]
    L.lh_scene_mesh_count.restype = C.c_uint32
    L.lh_scene_mesh_get.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(SceneMesh)]
    L.lh_scene_mesh_get.restype = C.c_int32
    L.lh_scene_instance_records.argtypes = [C.c_void_p, C.c_void_p]
    L.lh_scene_instance_records.restype = C.c_int32
    n = L.lh_scene_mesh_count(scene.handle)
    recs = []
    for i in range(n):
        m = SceneMesh()
        _check(L.lh_scene_mesh_get(scene.handle, i, C.byref(m)), "lh_scene_mesh_get")
        recs.append(m)
    inst = np.zeros(scene.desc.n_instances, np.uint32)
    _check(L.lh_scene_instance_records(scene.handle, inst.ctypes.data), "lh_scene_instance_records")
    return recs, inst


def _host_floats(addr, n):
    return np.ctypeslib.as_array((C.c_float * n).from_address(addr)).copy()


class DiffResolve:
    def __init__(self, renderer, scene, device="cuda"):
        import torch
        self.torch = torch
        self.renderer = renderer
        self.scene = scene
        from . import CONFIG_HDR_RGBA16F
        if renderer.config.flags & CONFIG_HDR_RGBA16F:
            raise ValueError("the differentiable resolve needs the RGBA32F HDR image")
        recs, inst = _scene_records(scene)
        if not recs or not recs[0].device_info:
            raise ValueError("scene is not uploaded")
        meshes = {}
        for r in recs:
            if r.mesh not in meshes:
                meshes[r.mesh] = r
        self.mesh_ids = sorted(meshes)
        pos, nrm, uvs, layout = [], [], [], []
        first = 0
        for m in self.mesh_ids:
            r = meshes[m]
            if not (r.flags & 4):
                raise ValueError("differentiation needs fp32 vertex attributes")
            hi = r.host_info
            hp = C.cast(hi, C.POINTER(C.c_uint64))
            pos.append(_host_floats(hp[0], r.vertices * 3))
            nrm.append(_host_floats(hp[2], r.vertices * 3))
            uvs.append(_host_floats(hp[3], r.vertices * 2))
            layout.append([r.vertices, first, r.device_positions, r.device_normals, r.device_uvs, 1])
            first += r.vertices
        self.mesh_layout = torch.tensor(np.array(layout, np.uint64).view(np.int64), dtype=torch.int64)
        self.record_layout = torch.tensor([[self.mesh_ids.index(r.mesh), r.device_info + 92] for r in recs],
                                          dtype=torch.int64)
        self.instance_record = torch.from_numpy(inst.astype(np.int64))
        bcf = [np.ctypeslib.as_array((C.c_float * 3).from_address(r.host_info + 92)).copy() for r in recs]
        self.positions = torch.from_numpy(np.concatenate(pos)).to(device).requires_grad_()
        self.normals = torch.from_numpy(np.concatenate(nrm)).to(device).requires_grad_()
        self.uvs = torch.from_numpy(np.concatenate(uvs)).to(device).requires_grad_()
        self.base_color_factor = torch.from_numpy(np.stack(bcf)).to(device).requires_grad_()
        # textures: the context's linear copies (what the kernels sample)
        tex, tex_layout = [], []
        for i in range(scene.desc.n_textures):
            addr, w, h = renderer.texture_linear(i)
            host = np.empty(w * h * 4, np.float32)
            _check(lib().lh_download(renderer.ctx, host.ctypes.data, addr, host.nbytes), "lh_download", renderer.ctx)
            tex.append(host)
            tex_layout.append([w * h, addr])
        self.texture_layout = torch.tensor(np.array(tex_layout, np.uint64).reshape(-1, 2).view(np.int64),
                                           dtype=torch.int64)
        self.texture_shapes = [(int(renderer.texture_linear(i)[2]), int(renderer.texture_linear(i)[1]))
                               for i in range(scene.desc.n_textures)]
        flat = np.concatenate(tex) if tex else np.zeros(0, np.float32)
        self.textures = torch.from_numpy(flat).to(device).requires_grad_()
        f = uniforms_fields(scene.uniforms)
        self.light_dir = torch.tensor(f["sun_dir"], dtype=torch.float32, device=device).requires_grad_()
        self.light_color = torch.tensor(f["sun_intensity"], dtype=torch.float32, device=device).requires_grad_()

    def parameters(self):
        return {"positions": self.positions, "normals": self.normals, "uvs": self.uvs,
                "base_color_factor": self.base_color_factor, "light_dir": self.light_dir,
                "light_color": self.light_color, "textures": self.textures}

    def texture_offset(self, index):
        """First float of texture `index` in `textures` (4 floats per texel)."""
        return 4 * int(self.texture_layout[:index, 0].sum())

    def texture_view(self, tensor, index):
        """[h, w, 4] view of texture `index` inside a tensor shaped like
        `textures` (the parameter itself or its gradient)."""
        h, w = self.texture_shapes[index]
        o = self.texture_offset(index)
        return tensor[o:o + 4 * w * h].view(h, w, 4)

    def __call__(self, uniforms=None):
        torch = self.torch
        u = uniforms if uniforms is not None else self.scene.uniforms
        ub = torch.from_numpy(np.frombuffer(bytes(u), np.uint8).copy())
        return extension().resolve(self.renderer.ctx.value, ub, self.mesh_layout, self.record_layout,
                                   self.instance_record, self.texture_layout, self.light_dir, self.light_color,
                                   self.positions, self.normals, self.uvs, self.base_color_factor, self.textures)
