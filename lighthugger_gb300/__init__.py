"""GB300 visibility pipeline: Python host mirror of the C ABI (include/lh/lh.h).

The reference drives its GPU passes from C++ (`render()`, src/rendering.cpp:28)
with a `Uniforms` struct per frame and device-address-linked scene buffers.
This module exposes the same operator boundary to Python through ctypes:

    scene = Scene(config_id=2, seed=20261205)    # seeded synthetic scene (host + device copy)
    r = Renderer(Config(width=1920, height=1080, shadow_size=1024, max_instances=4096))
    r.set_scene(scene)
    r.frame(scene.uniforms)                       # cull -> raster -> depth -> cascades -> shadows -> resolve
    vis = r.visibility()                          # numpy u64 [H, W]

The native library must be present (built by lighthugger_gb300.build); there
is no CPU fallback -- a missing library raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblh.so")

LH_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARGUMENT", 2: "CUDA", 3: "OUT_OF_MEMORY", 4: "CAPACITY", 5: "TIMEOUT",
                6: "NO_SCENE", 7: "UNSUPPORTED"}

FLAG_INSTANCE_OVERFLOW = 0x1
FLAG_DRAW_OVERFLOW = 0x2
FLAG_QUEUE_OVERFLOW = 0x4
FLAG_TIMEOUT = 0x8
FLAG_BAD_MESHLET = 0x10
FLAG_NO_DEPTH = 0x20
FLAG_SLOT_OVERFLOW = 0x40

WAIT_LOOKBACK, WAIT_GRID_BARRIER, WAIT_MBARRIER = 0, 1, 2

STAGES = ["clear", "cull_instances", "cull_meshlets", "raster", "depth_fit", "shadow_cull_instances",
          "shadow_cull_meshlets", "shadow_raster", "resolve"]

UNIFORMS_BYTES = 560
MISC_BYTES = 792
INSTANCE_BYTES = 112


class LHError(RuntimeError):
    def __init__(self, status, what, detail=""):
        super().__init__("%s failed: %s%s" % (what, STATUS_NAMES.get(status, status), (" (%s)" % detail) if detail else ""))
        self.status = status


class Config(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("shadow_size", C.c_uint32),
                ("max_instances", C.c_uint32), ("max_draws", C.c_uint32), ("max_big_triangles", C.c_uint32),
                ("max_probes", C.c_uint32), ("max_probe_pixels", C.c_uint32), ("device", C.c_int32),
                ("flags", C.c_uint32)]


class Texture(C.Structure):
    _fields_ = [("texels", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32), ("srgb", C.c_uint32),
                ("reserved", C.c_uint32)]


class FrameOut(C.Structure):
    _fields_ = [("visibility", C.c_uint64), ("hdr", C.c_uint64), ("shadow_maps", C.c_uint64),
                ("misc_storage", C.c_uint64), ("prefix_sums", C.c_uint64), ("meshlet_references", C.c_uint64),
                ("draw_calls", C.c_uint64), ("probe_visibility", C.c_uint64), ("prefix_sector_bytes", C.c_uint64),
                ("draw_call_section_bytes", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32),
                ("shadow_size", C.c_uint32), ("max_instances", C.c_uint32), ("max_draws", C.c_uint32),
                ("n_views", C.c_uint32), ("n_probes", C.c_uint32), ("reserved", C.c_uint32)]


class DeviceStatus(C.Structure):
    _fields_ = [("flags", C.c_uint32), ("n_views", C.c_uint32), ("visible_instances", C.c_uint32 * 40),
                ("candidate_meshlets", C.c_uint32 * 40), ("visible_opaque", C.c_uint32 * 40),
                ("visible_alpha_clip", C.c_uint32 * 40), ("big_triangles", C.c_uint32),
                ("clipped_triangles", C.c_uint32), ("fragments", C.c_uint32 * 2),
                ("occlusion", C.c_uint32 * 3)]


SCHEDULE_DEFAULT, SCHEDULE_PER_STAGE, SCHEDULE_PERSISTENT, SCHEDULE_PER_VIEW = 0, 1, 2, 3
CONFIG_HDR_RGBA16F = 1  # lh_config.flags: the HDR image in RGBA16F


class Tuning(C.Structure):
    _fields_ = [("small_px", C.c_uint32), ("medium_px", C.c_uint32), ("cull_blocks_per_sm", C.c_float),
                ("schedule", C.c_uint32), ("raster_batch", C.c_uint32), ("occlusion_px", C.c_uint32),
                ("chunk_rows", C.c_uint32 * 2), ("chunk_cols", C.c_uint32 * 2), ("backward_rows", C.c_uint32)]

    def as_dict(self):
        return {"small_px": self.small_px, "medium_px": self.medium_px, "cull_blocks_per_sm": self.cull_blocks_per_sm,
                "schedule": self.schedule, "raster_batch": self.raster_batch, "occlusion_px": self.occlusion_px,
                "chunk_rows": list(self.chunk_rows), "chunk_cols": list(self.chunk_cols),
                "backward_rows": self.backward_rows}


class MeshGrads(C.Structure):
    _fields_ = [("positions", C.c_uint64), ("normals", C.c_uint64), ("uvs", C.c_uint64),
                ("base_color_factor", C.c_uint64)]


class GradTargets(C.Structure):
    _fields_ = [("instance_grads", C.c_uint64), ("texture_grads", C.c_uint64), ("light_dir", C.c_uint64),
                ("light_color", C.c_uint64)]


class SceneParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("n_instances", C.c_uint32), ("n_probes", C.c_uint32),
                ("detail", C.c_float), ("quantized", C.c_uint32), ("reference_normal_transform", C.c_uint32),
                ("alpha_clip_materials", C.c_uint32), ("reserved", C.c_uint32 * 4)]


Uniforms = C.c_uint8 * UNIFORMS_BYTES


class SceneDesc(C.Structure):
    _fields_ = [("config_id", C.c_uint32), ("n_instances", C.c_uint32), ("n_meshes", C.c_uint32),
                ("n_textures", C.c_uint32), ("n_probes", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("shadow_size", C.c_uint32), ("total_meshlets", C.c_uint64), ("total_triangles", C.c_uint64),
                ("seed", C.c_uint64), ("host_instances", C.c_void_p), ("host_textures", C.POINTER(Texture)),
                ("device_instances", C.c_void_p), ("device_textures", C.POINTER(Texture)), ("uniforms", Uniforms),
                ("probes", C.c_void_p), ("device_bytes", C.c_uint64)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("yaw", C.c_float), ("pitch", C.c_float), ("fov_degrees", C.c_float),
                ("sun_latitude", C.c_float), ("sun_longitude", C.c_float), ("width", C.c_uint32),
                ("height", C.c_uint32), ("shadow_cam_distance", C.c_float), ("cascade_split_pow", C.c_float),
                ("num_instances", C.c_uint32)]


_lib = None


def lib():
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("native library %s is missing: run lighthugger_gb300.build.build()" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    L.lh_version.restype = C.c_uint32
    L.lh_create.argtypes = [C.POINTER(Config), C.POINTER(P)]
    L.lh_set_scene.argtypes = [P, P, C.c_uint32, C.POINTER(Texture), C.c_uint32]
    L.lh_frame.argtypes = [P, P, P, C.POINTER(FrameOut)]
    L.lh_frame_batched.argtypes = [P, P, P, C.c_uint32, P, C.POINTER(FrameOut)]
    L.lh_frame_graph.argtypes = [P, P, P, C.c_uint32, P, C.POINTER(FrameOut)]
    L.lh_frame_readback.argtypes = [P, P, P, P, C.POINTER(FrameOut)]
    L.lh_scene_from_mesh.argtypes = [P, P, P, C.c_uint32, P, C.c_uint32, P, C.c_uint32, P, C.POINTER(P)]
    L.lh_readback_wait.argtypes = [P]
    L.lh_get_outputs.argtypes = [P, C.POINTER(FrameOut)]
    L.lh_read_status.argtypes = [P, C.POINTER(DeviceStatus)]
    L.lh_download.argtypes = [P, P, C.c_uint64, C.c_size_t]
    L.lh_last_error.argtypes = [P]
    L.lh_last_error.restype = C.c_char_p
    L.lh_destroy.argtypes = [P]
    L.lh_destroy.restype = None
    L.lh_resolve_backward.argtypes = [P, C.c_uint64, C.POINTER(GradTargets), P]
    L.lh_frame_graph_backward.argtypes = [P, P, P, C.c_uint32, C.c_uint64, C.POINTER(GradTargets), P,
                                          C.POINTER(FrameOut)]
    L.lh_display_transform.argtypes = [P, C.c_uint64, C.c_uint64, P]
    L.lh_set_profiling.argtypes = [P, C.c_int]
    L.lh_get_stage_times.argtypes = [P, C.POINTER(C.c_float), C.c_uint32]
    L.lh_set_tuning.argtypes = [P, C.POINTER(Tuning)]
    L.lh_get_tuning.argtypes = [P, C.POINTER(Tuning)]
    L.lh_scene_create.argtypes = [C.c_uint32, C.c_uint64, C.POINTER(SceneParams), C.POINTER(P)]
    L.lh_scene_describe.argtypes = [P, C.POINTER(SceneDesc)]
    L.lh_scene_upload.argtypes = [P, C.c_int]
    L.lh_scene_save.argtypes = [P, C.c_char_p]
    L.lh_scene_load.argtypes = [C.c_char_p, C.POINTER(P)]
    L.lh_scene_destroy.argtypes = [P]
    L.lh_scene_destroy.restype = None
    L.lh_make_uniforms.argtypes = [C.POINTER(Camera), C.POINTER(Uniforms)]
    L.lh_cull_instances_noalloc.argtypes = [P, C.c_uint32, P, P, C.c_uint32, P, P]
    L.lh_check_bounded_wait.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, P, P]
    L.lh_probe_red_u64.argtypes = [P, C.c_uint64, C.c_uint32, C.c_uint32, P]
    L.lh_get_texture_linear.argtypes = [P, C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32)]
    for name in ("lh_create", "lh_set_scene", "lh_frame", "lh_frame_batched", "lh_frame_graph", "lh_get_outputs",
                 "lh_read_status",
                 "lh_download", "lh_resolve_backward", "lh_frame_graph_backward", "lh_display_transform", "lh_set_profiling", "lh_get_stage_times", "lh_set_tuning", "lh_get_tuning", "lh_scene_create", "lh_scene_describe", "lh_scene_save", "lh_scene_load",
                 "lh_scene_upload", "lh_make_uniforms", "lh_cull_instances_noalloc", "lh_check_bounded_wait",
                 "lh_get_texture_linear", "lh_probe_red_u64"):
        getattr(L, name).restype = C.c_int32
    _lib = L
    return L


def _check(st, what, ctx=None):
    if st != LH_OK:
        detail = ""
        if ctx:
            detail = (lib().lh_last_error(ctx) or b"").decode(errors="replace")
        raise LHError(st, what, detail)


def default_seed(config_id):
    return 20261203 + config_id


class Scene:
    """A seeded synthetic scene (lh_scene_create); `upload()` makes the device copy."""

    def __init__(self, config_id, seed=None, **params):
        self.config_id = config_id
        self.seed = default_seed(config_id) if seed is None else seed
        p = SceneParams()
        for k, v in params.items():
            if v is not None:
                setattr(p, k, v)
        h = C.c_void_p()
        _check(lib().lh_scene_create(config_id, self.seed, C.byref(p), C.byref(h)), "lh_scene_create")
        self.handle = h
        self.params = params
        self._describe()

    @classmethod
    def from_mesh(cls, positions, indices, transforms, uniforms, normals=None, uvs=None):
        """A scene of one caller mesh (lh_scene_from_mesh): positions float
        [n, 3], indices [m, 3], transforms [k, 4, 4] (row-major numpy, applied
        to column vectors), camera Uniforms."""
        pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
        # lh_mat4 is column major: the transpose of the row-major matrix
        tr = np.ascontiguousarray(np.transpose(np.asarray(transforms, dtype=np.float32).reshape(-1, 4, 4), (0, 2, 1)))
        nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        uv = None if uvs is None else np.ascontiguousarray(uvs, dtype=np.float32).reshape(-1, 2)
        ptr = lambda a: None if a is None else a.ctypes.data
        h = C.c_void_p()
        _check(lib().lh_scene_from_mesh(ptr(pos), ptr(nrm), ptr(uv), len(pos), ptr(idx), len(idx), ptr(tr), len(tr),
                                        C.byref(uniforms), C.byref(h)), "lh_scene_from_mesh")
        self = cls.__new__(cls)
        self.config_id = 0
        self.seed = 0
        self.handle = h
        self.params = {}
        self._describe()
        return self

    def save(self, path):
        """Write the scene's host copy to a dump file (lh_scene_save)."""
        _check(lib().lh_scene_save(self.handle, os.fsencode(path)), "lh_scene_save")

    @classmethod
    def load(cls, path):
        """A scene read back from a dump file (lh_scene_load)."""
        h = C.c_void_p()
        _check(lib().lh_scene_load(os.fsencode(path), C.byref(h)), "lh_scene_load")
        self = cls.__new__(cls)
        self.handle = h
        self.params = {}
        self._describe()
        self.config_id = self.desc.config_id
        self.seed = self.desc.seed
        return self

    def _describe(self):
        d = SceneDesc()
        _check(lib().lh_scene_describe(self.handle, C.byref(d)), "lh_scene_describe")
        self.desc = d

    def upload(self, device=0):
        _check(lib().lh_scene_upload(self.handle, device), "lh_scene_upload")
        self._describe()
        return self

    @property
    def uniforms(self):
        u = Uniforms()
        C.memmove(u, self.desc.uniforms, UNIFORMS_BYTES)
        return u

    def probe_uniforms(self):
        n = self.desc.n_probes
        arr = (Uniforms * max(n, 1))()
        if n:
            C.memmove(arr, self.desc.probes, UNIFORMS_BYTES * n)
        return arr, n

    def host_instances_ptr(self):
        return self.desc.host_instances

    def close(self):
        if getattr(self, "handle", None):
            lib().lh_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_uniforms(position, yaw, pitch, fov_degrees, width, height, num_instances, sun_latitude=-5.6,
                  sun_longitude=1.37, shadow_cam_distance=1024.0, cascade_split_pow=3.0):
    """Host uniform math of src/main.cpp:734-760 (lookAt + infinite reverse-Z)."""
    cam = Camera()
    cam.position[:] = position
    cam.yaw, cam.pitch, cam.fov_degrees = yaw, pitch, fov_degrees
    cam.sun_latitude, cam.sun_longitude = sun_latitude, sun_longitude
    cam.width, cam.height = width, height
    cam.shadow_cam_distance, cam.cascade_split_pow = shadow_cam_distance, cascade_split_pow
    cam.num_instances = num_instances
    u = Uniforms()
    _check(lib().lh_make_uniforms(C.byref(cam), C.byref(u)), "lh_make_uniforms")
    return u


def uniforms_fields(u):
    """Numpy view of the matrix / vector fields of a Uniforms blob."""
    b = np.frombuffer(bytes(u), dtype=np.uint8)
    f = b[:448].view(np.float32).reshape(7, 4, 4)
    names = ["combined_perspective_view", "inv_perspective_view", "view", "initial_view", "perspective",
             "perspective_inverse", "view_inverse"]
    out = {n: f[i] for i, n in enumerate(names)}
    v = b[496:532].view(np.float32)
    out["camera_pos"], out["sun_dir"], out["sun_intensity"] = v[0:3], v[3:6], v[6:9]
    out["num_instances"] = int(b[532:536].view(np.uint32)[0])
    out["window_size"] = tuple(int(x) for x in b[536:544].view(np.uint32))
    out["shadow_cam_distance"], out["cascade_split_pow"] = (float(x) for x in b[544:552].view(np.float32))
    return out


class Renderer:
    """One lh_ctx: owns scratch and outputs; `frame()` enqueues one frame."""

    def __init__(self, config):
        h = C.c_void_p()
        _check(lib().lh_create(C.byref(config), C.byref(h)), "lh_create")
        self.ctx = h
        self.config = config
        self.out = FrameOut()
        self.stream = None

    def set_scene(self, scene):
        d = scene.desc
        if not d.device_instances:
            raise ValueError("scene is not uploaded")
        _check(lib().lh_set_scene(self.ctx, d.device_instances, d.n_instances, d.device_textures, d.n_textures),
               "lh_set_scene", self.ctx)
        self.scene = scene

    def set_tuning(self, small_px=None, medium_px=None, cull_blocks_per_sm=None, schedule=None, raster_batch=None,
                   occlusion_px=None, chunk_rows=None, chunk_cols=None, backward_rows=None):
        """Set the given launch-shape knobs (lh_tuning); chunk_rows / chunk_cols
        are pairs (visibility pass, shadow pass)."""
        t = self.tuning()
        if occlusion_px is not None:
            t.occlusion_px = occlusion_px
        if chunk_rows is not None:
            t.chunk_rows[0], t.chunk_rows[1] = chunk_rows
        if chunk_cols is not None:
            t.chunk_cols[0], t.chunk_cols[1] = chunk_cols
        if backward_rows is not None:
            t.backward_rows = backward_rows
        if schedule is not None:
            t.schedule = schedule
        if raster_batch is not None:
            t.raster_batch = raster_batch
        if small_px is not None:
            t.small_px = small_px
        if medium_px is not None:
            t.medium_px = medium_px
        if cull_blocks_per_sm is not None:
            t.cull_blocks_per_sm = cull_blocks_per_sm
        _check(lib().lh_set_tuning(self.ctx, C.byref(t)), "lh_set_tuning", self.ctx)

    def set_profiling(self, enable=True):
        _check(lib().lh_set_profiling(self.ctx, 1 if enable else 0), "lh_set_profiling", self.ctx)

    def stage_times(self):
        ms = (C.c_float * len(STAGES))()
        _check(lib().lh_get_stage_times(self.ctx, ms, len(STAGES)), "lh_get_stage_times", self.ctx)
        return dict(zip(STAGES, [float(x) for x in ms]))

    def tuning(self):
        t = Tuning()
        _check(lib().lh_get_tuning(self.ctx, C.byref(t)), "lh_get_tuning", self.ctx)
        return t

    def frame(self, uniforms, stream=None):
        s = stream if stream is not None else self.stream
        _check(lib().lh_frame(self.ctx, C.byref(uniforms), s, C.byref(self.out)), "lh_frame", self.ctx)
        return self.out

    def frame_readback(self, uniforms, host_hdr_ptr, stream=None):
        """lh_frame with the HDR image copied to host memory at host_hdr_ptr,
        pipelined with the next frame: when this returns, the buffer given to
        the previous call holds that frame (readback_wait() for the last)."""
        s = stream if stream is not None else self.stream
        _check(lib().lh_frame_readback(self.ctx, C.byref(uniforms), host_hdr_ptr, s, C.byref(self.out)),
               "lh_frame_readback", self.ctx)
        return self.out

    def readback_wait(self):
        _check(lib().lh_readback_wait(self.ctx), "lh_readback_wait", self.ctx)

    def frame_batched(self, uniforms, probes, n_probes, stream=None):
        s = stream if stream is not None else self.stream
        _check(lib().lh_frame_batched(self.ctx, C.byref(uniforms), probes if n_probes else None, n_probes, s,
                                      C.byref(self.out)), "lh_frame_batched", self.ctx)
        return self.out

    def frame_graph(self, uniforms, probes=None, n_probes=0, stream=None):
        s = stream if stream is not None else self.stream
        _check(lib().lh_frame_graph(self.ctx, C.byref(uniforms), probes if n_probes else None, n_probes, s,
                                    C.byref(self.out)), "lh_frame_graph", self.ctx)
        return self.out

    def frame_graph_backward(self, uniforms, probes, n_probes, grad_ptr, targets, stream=None):
        """The batched frame and the resolve adjoint of its main view, replayed
        from one captured CUDA graph."""
        s = stream if stream is not None else self.stream
        _check(lib().lh_frame_graph_backward(self.ctx, C.byref(uniforms), probes if n_probes else None, n_probes,
                                             grad_ptr, C.byref(targets), s, C.byref(self.out)),
               "lh_frame_graph_backward", self.ctx)
        return self.out

    def texture_linear(self, index):
        """(device address, width, height) of the context's linear float4
        copy of texture `index` (what the frames and the adjoint sample)."""
        a, w, h = C.c_uint64(), C.c_uint32(), C.c_uint32()
        _check(lib().lh_get_texture_linear(self.ctx, index, C.byref(a), C.byref(w), C.byref(h)),
               "lh_get_texture_linear", self.ctx)
        return int(a.value), int(w.value), int(h.value)

    def display_transform(self, out_ptr, lut_ptr=0, stream=None):
        """RGBA8 display image of the last frame into device buffer out_ptr
        (uchar4[h][w]); lut_ptr: float4[48][48][48] or 0 for the stand-in."""
        s = stream if stream is not None else self.stream
        _check(lib().lh_display_transform(self.ctx, lut_ptr, out_ptr, s), "lh_display_transform", self.ctx)

    def status(self):
        st = DeviceStatus()
        _check(lib().lh_read_status(self.ctx, C.byref(st)), "lh_read_status", self.ctx)
        return st

    def download(self, device_ptr, nbytes, dtype=np.uint8):
        buf = np.empty(nbytes, dtype=np.uint8)
        if nbytes:
            _check(lib().lh_download(self.ctx, buf.ctypes.data, device_ptr, nbytes), "lh_download", self.ctx)
        return buf.view(dtype)

    # ---- typed result accessors (synchronising)
    def visibility(self):
        o = self.out
        return self.download(o.visibility, o.width * o.height * 8, np.uint64).reshape(o.height, o.width)

    def hdr(self):
        """The HDR image as float32 [h, w, 4] (float16 with CONFIG_HDR_RGBA16F)."""
        o = self.out
        if self.config.flags & CONFIG_HDR_RGBA16F:
            return self.download(o.hdr, o.width * o.height * 8, np.float16).reshape(o.height, o.width, 4)
        return self.download(o.hdr, o.width * o.height * 16, np.float32).reshape(o.height, o.width, 4)

    def shadow_maps(self):
        o = self.out
        S = o.shadow_size
        return self.download(o.shadow_maps, 4 * S * S * 4, np.float32).reshape(4, S, S)

    def misc(self):
        return self.download(self.out.misc_storage, MISC_BYTES)

    def prefix_sector(self, view):
        o = self.out
        raw = self.download(o.prefix_sums + view * o.prefix_sector_bytes, o.prefix_sector_bytes)
        return raw

    def draw_section(self, view):
        o = self.out
        return self.download(o.draw_calls + view * o.draw_call_section_bytes, o.draw_call_section_bytes)

    def meshlet_references(self, view):
        o = self.out
        n = 2 * o.max_draws
        return self.download(o.meshlet_references + view * n * 8, n * 8)

    def probe_visibility(self, probes, n_probes):
        """List of u64 [h, w] arrays, one per probe (packed back to back, 32-pixel aligned)."""
        out, off = [], 0
        for p in range(n_probes):
            f = uniforms_fields(probes[p])
            w, h = f["window_size"]
            a = self.download(self.out.probe_visibility + off * 8, w * h * 8, np.uint64).reshape(h, w)
            out.append(a)
            off += (w * h + 31) // 32 * 32
        return out

    def close(self):
        if getattr(self, "ctx", None):
            lib().lh_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
