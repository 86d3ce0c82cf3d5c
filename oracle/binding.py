"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
as the checker; the product path never imports it.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

STAGE_CULL, STAGE_RASTER, STAGE_DEPTH, STAGE_SHADOW, STAGE_RESOLVE = 1, 2, 4, 8, 16
STAGE_ALL = 31
STAGE_NAMES = ["cull", "raster", "depth_fit", "shadow_cull", "shadow_raster", "resolve", "total", "threads"]


class FrameDesc(C.Structure):
    _fields_ = [("instances", C.c_void_p), ("n_instances", C.c_uint32), ("textures", C.c_void_p),
                ("n_textures", C.c_uint32), ("uniforms", C.c_void_p), ("shadow_size", C.c_uint32),
                ("max_instances", C.c_uint32), ("max_draws", C.c_uint32), ("threads", C.c_int32),
                ("stages", C.c_uint32), ("texture_linear", C.c_void_p)]


class FrameOut(C.Structure):
    _fields_ = [("prefix_sums", C.c_void_p), ("meshlet_references", C.c_void_p), ("draw_calls", C.c_void_p),
                ("visibility", C.c_void_p), ("shadow_maps", C.c_void_p), ("misc", C.c_void_p), ("hdr", C.c_void_p),
                ("stage_ms", C.c_double * 8), ("flags", C.c_uint32), ("reserved", C.c_uint32),
                ("stats", C.c_uint64 * 16)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.lho_frame.argtypes = [C.POINTER(FrameDesc), C.POINTER(FrameOut)]
        L.lho_frame.restype = C.c_int
        L.lho_raster_triangle.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p]
        L.lho_raster_triangle.restype = C.c_int
        L.lho_raster_triangle_alpha.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                                C.c_uint32, C.c_uint32, C.c_void_p]
        L.lho_raster_triangle_alpha.restype = C.c_int
        L.lho_display_transform.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                            C.c_uint32, C.c_void_p]
        L.lho_display_transform.restype = C.c_int
        L.lho_resolve_f64.argtypes = [C.POINTER(FrameDesc), C.POINTER(FrameOut), C.c_void_p]
        L.lho_resolve_f64.restype = C.c_int
        L.lho_resolve_f64_pixels.argtypes = [C.POINTER(FrameDesc), C.POINTER(FrameOut), C.c_void_p, C.c_uint32,
                                             C.c_void_p]
        L.lho_resolve_f64_pixels.restype = C.c_int
        _lib = L
    return _lib


def align16(n):
    return (n + 15) // 16 * 16


class OracleFrame:
    """Result buffers of one oracle frame, laid out as lh_frame_out documents."""

    def __init__(self, width, height, shadow_size, max_instances, max_draws):
        self.W, self.H, self.S = width, height, shadow_size
        self.max_instances, self.max_draws = max_instances, max_draws
        self.sector_bytes = align16(8 + 8 * max_instances)
        self.draw_bytes = align16(8 + 16 * 2 * max_draws)
        # the oracle uses unaligned section strides (8 + 8*cap, 8 + 32*max_draws)
        self.o_sector = 8 + 8 * max_instances
        self.o_draw = 8 + 16 * 2 * max_draws
        self.prefix = np.zeros(5 * self.o_sector, np.uint8)
        self.refs = np.zeros(5 * 2 * max_draws * 8, np.uint8)
        self.draws = np.zeros(5 * self.o_draw, np.uint8)
        self.vis = np.zeros((height, width), np.uint64)
        self.shadow = np.zeros((4, shadow_size, shadow_size), np.float32)
        self.misc = np.zeros(792, np.uint8)
        self.hdr = np.zeros((height, width, 4), np.float32)
        self.out = FrameOut()
        self.out.prefix_sums = self.prefix.ctypes.data
        self.out.meshlet_references = self.refs.ctypes.data
        self.out.draw_calls = self.draws.ctypes.data
        self.out.visibility = self.vis.ctypes.data
        self.out.shadow_maps = self.shadow.ctypes.data
        self.out.misc = self.misc.ctypes.data
        self.out.hdr = self.hdr.ctypes.data

    def sector(self, view):
        return self.prefix[view * self.o_sector:(view + 1) * self.o_sector]

    def draw_section(self, view):
        return self.draws[view * self.o_draw:(view + 1) * self.o_draw]

    def meshlet_references(self, view):
        n = 2 * self.max_draws * 8
        return self.refs[view * n:(view + 1) * n]

    @property
    def stage_ms(self):
        return dict(zip(STAGE_NAMES, list(self.out.stage_ms)))

    @property
    def raster_stats(self):
        names = ["triangles", "fragments", "bbox_le4", "bbox_le64", "bbox_le4096", "bbox_gt4096", "clipped",
                 "max_meshlet_fragments"]
        s = list(self.out.stats)
        return {"visibility": dict(zip(names, s[:8])), "shadow": dict(zip(names, s[8:]))}

    @property
    def flags(self):
        return int(self.out.flags)


def run_frame(host_instances, n_instances, host_textures, n_textures, uniforms, shadow_size, max_instances, max_draws,
              threads=0, stages=STAGE_ALL):
    """Run the oracle over a host scene (host addresses in the records)."""
    import lighthugger_gb300 as lh
    f = lh.uniforms_fields(uniforms)
    W, H = f["window_size"]
    fr = OracleFrame(W, H, shadow_size, max_instances, max_draws)
    d = FrameDesc()
    d.instances = host_instances
    d.n_instances = n_instances
    d.textures = C.cast(host_textures, C.c_void_p).value if host_textures else None
    d.n_textures = n_textures
    ubuf = (C.c_uint8 * len(bytes(uniforms))).from_buffer_copy(bytes(uniforms))
    fr._ubuf = ubuf
    d.uniforms = C.addressof(ubuf)
    d.shadow_size = shadow_size
    d.max_instances = max_instances
    d.max_draws = max_draws
    d.threads = threads
    d.stages = stages
    st = lib().lho_frame(C.byref(d), C.byref(fr.out))
    if st != 0:
        raise RuntimeError("lho_frame failed: %d" % st)
    fr.desc = d
    return fr


def run_scene(scene, shadow_size=None, max_instances=None, max_draws=None, threads=0, stages=STAGE_ALL,
              uniforms=None):
    d = scene.desc
    return run_frame(d.host_instances, d.n_instances, d.host_textures, d.n_textures,
                     uniforms if uniforms is not None else scene.uniforms,
                     shadow_size or d.shadow_size, max_instances or max(1024, d.n_instances),
                     max_draws or 200000, threads, stages)


def resolve_f64(frame):
    out = np.zeros((frame.H, frame.W, 4), np.float64)
    st = lib().lho_resolve_f64(C.byref(frame.desc), C.byref(frame.out), out.ctypes.data)
    if st != 0:
        raise RuntimeError("lho_resolve_f64 failed: %d" % st)
    return out


def resolve_f64_pixels(frame, xy):
    """FP64 resolve of the listed pixels (int array [n, 2] of x, y): [n, 4]."""
    xy = np.ascontiguousarray(xy, dtype=np.uint32).reshape(-1, 2)
    out = np.zeros((len(xy), 4), np.float64)
    st = lib().lho_resolve_f64_pixels(C.byref(frame.desc), C.byref(frame.out), xy.ctypes.data, len(xy),
                                      out.ctypes.data)
    if st != 0:
        raise RuntimeError("lho_resolve_f64_pixels failed: %d" % st)
    return out


def set_linear_textures(frame, textures):
    """Sample the given linear RGBA float32 arrays (one per texture, [h, w, 4]
    or flat; None keeps that texture's RGBA8 texels) in the frame's later
    float64 resolves.  The arrays are kept alive by the frame and may be
    changed in place between resolves."""
    arrs = [None if t is None else np.ascontiguousarray(t, dtype=np.float32) for t in textures]
    table = (C.c_void_p * max(1, len(arrs)))(*[None if a is None else a.ctypes.data for a in arrs])
    frame._linear = (arrs, table)
    frame.desc.texture_linear = C.cast(table, C.c_void_p)
    return arrs


def raster_triangle(clip, tri_id, kind, width, height, target=None):
    """Rasterise one clip-space triangle (3x4 floats) with the pipeline's rules."""
    clip = np.ascontiguousarray(clip, dtype=np.float32).reshape(12)
    if target is None:
        target = np.zeros((height, width), np.uint64) if kind == 0 else np.full((height, width), 0x3F800000, np.uint64)
    st = lib().lho_raster_triangle(clip.ctypes.data, tri_id, kind, width, height, target.ctypes.data)
    if st != 0:
        raise RuntimeError("lho_raster_triangle failed: %d" % st)
    return target


class _Texture(C.Structure):
    """lh_texture (include/lh/lh.h)."""
    _fields_ = [("texels", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32), ("srgb", C.c_uint32),
                ("reserved", C.c_uint32)]


def raster_triangle_alpha(clip, uv, texels, tex_w, tex_h, tri_id, kind, width, height, target=None):
    """Rasterise one alpha-clip triangle: clip (3x4), per-vertex uv (3x2),
    RGBA8 texels (tex_h x tex_w x 4, linear)."""
    clip = np.ascontiguousarray(clip, dtype=np.float32).reshape(12)
    uv = np.ascontiguousarray(uv, dtype=np.float32).reshape(6)
    texels = np.ascontiguousarray(texels, dtype=np.uint8)
    tex = _Texture(texels=texels.ctypes.data, width=tex_w, height=tex_h, srgb=0)
    if target is None:
        target = np.zeros((height, width), np.uint64) if kind == 0 else np.full((height, width), 0x3F800000, np.uint64)
    st = lib().lho_raster_triangle_alpha(clip.ctypes.data, uv.ctypes.data, C.byref(tex), tri_id, kind, width, height,
                                         target.ctypes.data)
    if st != 0:
        raise RuntimeError("lho_raster_triangle_alpha failed: %d" % st)
    return target


def display_transform(hdr, lut=None, shadow_maps=None, debug_shadowmaps=0):
    """RGBA8 display image of a float HDR image [h, w, 4] (lut: float32
    [48, 48, 48, 4] or None for the identity stand-in)."""
    hdr = np.ascontiguousarray(hdr, np.float32)
    H, W = hdr.shape[:2]
    out = np.zeros((H, W, 4), np.uint8)
    lut_p = np.ascontiguousarray(lut, np.float32) if lut is not None else None
    sm = np.ascontiguousarray(shadow_maps, np.float32) if shadow_maps is not None else None
    S = sm.shape[-1] if sm is not None else 0
    st = lib().lho_display_transform(hdr.ctypes.data, W, H, lut_p.ctypes.data if lut_p is not None else None,
                                     sm.ctypes.data if sm is not None else None, S, debug_shadowmaps, out.ctypes.data)
    if st != 0:
        raise RuntimeError("lho_display_transform failed: %d" % st)
    return out
