"""ctypes mirror of include/rosy_gb300.h and marshalling of a Scene into it."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import scene as sc


class RzVertex(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("normal", C.c_float * 3), ("tangent", C.c_float * 4),
                ("color", C.c_float * 4), ("uv", C.c_float * 2)]


class RzMesh(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("position_count", C.c_uint32),
                ("index_count", C.c_uint32), ("indices", C.c_void_p)]


class RzTexture(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("levels", C.c_uint32),
                ("image_type", C.c_uint32), ("texels", C.c_void_p), ("format", C.c_uint32),
                ("reserved", C.c_uint32)]


TEXELS_RGBA8 = 0
TEXELS_BC7 = 1


class RzConfig(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("shadow_map_size", C.c_uint32),
                ("samples", C.c_uint32), ("device", C.c_int32), ("queue_chunks", C.c_uint32),
                ("reserved", C.c_uint32 * 2)]


class RzDrawConfig(C.Structure):
    _fields_ = [("cull_enabled", C.c_uint32), ("reverse_winding_order_enabled", C.c_uint32),
                ("depth_bias_enabled", C.c_uint32), ("depth_bias_constant", C.c_float),
                ("depth_bias_clamp", C.c_float), ("depth_bias_slope_factor", C.c_float),
                ("pcf_mode", C.c_uint32), ("shadow_cascades", C.c_uint32)]


class RzView(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("shadow_map_size", C.c_uint32), ("draw_config", RzDrawConfig)]


class RzTuning(C.Structure):
    _fields_ = [("chunk_stamps", C.c_uint32), ("small_extent", C.c_uint32), ("queue_chunks", C.c_uint32),
                ("batched", C.c_uint32)]


class RzFrameOut(C.Structure):
    _fields_ = [("color_rgba8", C.c_void_p), ("depth_f32", C.c_void_p), ("visibility_u64", C.c_void_p),
                ("shadow_map_f32", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("shadow_map_size", C.c_uint32), ("triangle_id_base", C.c_uint32)]


class RzGbuffer(C.Structure):
    _fields_ = [("color_rgba8", C.c_void_p), ("depth_f32", C.c_void_p), ("albedo_rgba8", C.c_void_p),
                ("normal_oct_f16x2", C.c_void_p), ("sources_u16", C.c_void_p), ("width", C.c_uint32),
                ("height", C.c_uint32)]


class RzRsyInfo(C.Structure):
    _fields_ = [("mesh_count", C.c_uint32), ("material_count", C.c_uint32), ("sampler_count", C.c_uint32),
                ("image_count", C.c_uint32), ("node_count", C.c_uint32), ("scene_count", C.c_uint32),
                ("root_scene", C.c_uint32), ("object_count", C.c_uint32), ("surface_count", C.c_uint32),
                ("static_object_count", C.c_uint32), ("coordinate_system", C.c_float * 16)]


class RzDdsInfo(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("levels", C.c_uint32),
                ("dxgi_format", C.c_uint32), ("supports_alpha", C.c_uint32), ("reserved", C.c_uint32),
                ("data_bytes", C.c_uint64), ("data", C.c_void_p)]


class RzStats(C.Structure):
    _fields_ = [("draw_call_count", C.c_uint32), ("triangle_count", C.c_uint32),
                ("shadow_setup_records", C.c_uint32), ("camera_setup_records", C.c_uint32),
                ("shadow_stamps", C.c_uint64), ("camera_stamps", C.c_uint64),
                ("error_flags", C.c_uint32), ("kernel_launches", C.c_uint32)]


assert C.sizeof(RzVertex) == 64
assert C.sizeof(RzView) == 48
assert C.sizeof(RzMesh) == 24
assert C.sizeof(RzTexture) == 32
assert C.sizeof(RzDdsInfo) == 40


def ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def texel_bytes(width: int, height: int, levels: int, fmt: int) -> int:
    """Bytes of a texture's level chain: 4 per texel (RGBA8) or 16 per 4 x 4 block (BC7)."""
    n = 0
    for l in range(levels):
        w, h = max(1, width >> l), max(1, height >> l)
        n += max(1, (w + 3) // 4) * max(1, (h + 3) // 4) * 16 if fmt == TEXELS_BC7 else w * h * 4
    return n


class Marshalled:
    """Keeps the numpy/ctypes buffers of one scene alive while C code uses them."""

    def __init__(self, s: "sc.Scene"):
        self.scene = s
        self.vertices = np.ascontiguousarray(s.vertices, np.float32)
        self.indices = np.ascontiguousarray(s.indices, np.uint32)
        self.mesh_table = np.ascontiguousarray(np.asarray(s.meshes, np.uint32).reshape(-1, 4))
        self.meshes = (RzMesh * len(s.meshes))()
        for i, (vo, vc, io, ic) in enumerate(s.meshes):
            # the library reads through these pointers: every range must lie inside its array
            if not (0 <= vo and vo + vc <= len(self.vertices) and 0 <= io and io + ic <= len(self.indices)):
                raise ValueError(f"mesh {i} lies outside the vertex or index array")
            self.meshes[i].positions = ptr(self.vertices) + int(vo) * 64
            self.meshes[i].position_count = int(vc)
            self.meshes[i].index_count = int(ic)
            self.meshes[i].indices = ptr(self.indices) + int(io) * 4
        self.objects = np.ascontiguousarray(s.objects, np.float32)
        self.surfaces = np.ascontiguousarray(s.surfaces)
        self.materials = np.ascontiguousarray(s.materials)
        self.samplers = np.ascontiguousarray(s.samplers)
        self.tex_data = [np.ascontiguousarray(t.texels, np.uint8) for t in s.textures]
        self.textures = (RzTexture * max(1, len(s.textures)))()
        for i, t in enumerate(s.textures):
            self.textures[i].width = t.width
            self.textures[i].height = t.height
            self.textures[i].levels = t.levels
            self.textures[i].image_type = t.image_type
            self.textures[i].texels = ptr(self.tex_data[i])
            self.textures[i].format = getattr(t, "format", TEXELS_RGBA8)
            if 0 < t.width and 0 < t.height and 0 < t.levels <= 16 and \
                    self.tex_data[i].nbytes < texel_bytes(t.width, t.height, t.levels, self.textures[i].format):
                raise ValueError(f"texture {i} holds fewer bytes than its level chain")
        self.scene_rec = np.ascontiguousarray(s.scene)
        dbg = getattr(s, "debug_objects", None)
        self.debug_objects = None if dbg is None else np.ascontiguousarray(dbg, sc.DEBUG_OBJECT_DTYPE)
        self.draw_config = np.ascontiguousarray(s.draw_config)

    @property
    def n_textures(self) -> int:
        return len(self.scene.textures)
