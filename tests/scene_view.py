"""Read a host scene (records linked by host addresses) into numpy arrays."""
import ctypes as C

import numpy as np

MESHINFO_DTYPE = np.dtype([("positions", "<u8"), ("indices", "<u8"), ("normals", "<u8"), ("uvs", "<u8"),
                           ("micro_indices", "<u8"), ("meshlets", "<u8"), ("num_meshlets", "<u2"), ("flags", "u1"),
                           ("pad", "u1"), ("bounding_sphere", "<f4", 4), ("texture_scale", "<f4", 2),
                           ("texture_offset", "<f4", 2), ("base_color_texture_index", "<u2"),
                           ("metallic_roughness_texture_index", "<u2"), ("normal_texture_index", "<u2"),
                           ("pad2", "<u2"), ("base_color_factor", "<f4", 3)])
INSTANCE_DTYPE = np.dtype([("transform", "<f4", (4, 4)), ("mesh_info_address", "<u8"),
                           ("normal_transform", "<f4", (3, 3)), ("pad", "<u4")])
MESHLET_DTYPE = np.dtype([("cone_apex", "<f4", 3), ("cone_axis", "<f4", 3), ("cone_cutoff", "<f4"),
                          ("bounding_sphere", "<f4", 4), ("triangle_offset", "<u4"), ("index_offset", "<u4"),
                          ("triangle_count", "u1"), ("index_count", "u1"), ("pad", "<u2")])
assert MESHINFO_DTYPE.itemsize == 104 and INSTANCE_DTYPE.itemsize == 112 and MESHLET_DTYPE.itemsize == 56

FLAG_32 = 1
FLAG_ALPHA = 2
FLAG_FP32 = 4


def read(addr, nbytes):
    return np.frombuffer(C.string_at(addr, nbytes), dtype=np.uint8)


def instances(scene):
    d = scene.desc
    return read(d.host_instances, d.n_instances * 112).view(INSTANCE_DTYPE)


def mesh_info(addr):
    return read(addr, 104).view(MESHINFO_DTYPE)[0]


class Mesh:
    """Arrays of one MeshInfo (positions as float in shader space)."""

    def __init__(self, mi):
        self.mi = mi
        self.n_meshlets = int(mi["num_meshlets"])
        self.meshlets = read(int(mi["meshlets"]), self.n_meshlets * 56).view(MESHLET_DTYPE)
        m = self.meshlets
        n_idx = int((m["index_offset"].astype(np.int64) + m["index_count"]).max())
        self.index_bytes = 4 if int(mi["flags"]) & FLAG_32 else 2
        self.indices = read(int(mi["indices"]), n_idx * self.index_bytes).view(
            np.uint32 if self.index_bytes == 4 else np.uint16).astype(np.int64)
        n_micro = int((m["triangle_offset"].astype(np.int64) + 3 * m["triangle_count"].astype(np.int64)).max())
        self.micro = read(int(mi["micro_indices"]), n_micro)
        n_vert = int(self.indices.max()) + 1
        self.fp32 = bool(int(mi["flags"]) & FLAG_FP32)
        if self.fp32:
            self.positions = read(int(mi["positions"]), n_vert * 12).view(np.float32).reshape(-1, 3).astype(np.float64)
        else:
            self.positions = read(int(mi["positions"]), n_vert * 6).view(np.uint16).reshape(-1, 3).astype(np.float64)

    def meshlet_triangles(self, k):
        m = self.meshlets[k]
        off, nt = int(m["triangle_offset"]), int(m["triangle_count"])
        micro = self.micro[off:off + 3 * nt].reshape(nt, 3).astype(np.int64)
        return micro, self.indices[int(m["index_offset"]) + micro]
