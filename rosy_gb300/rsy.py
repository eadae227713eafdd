"""Rosy .rsy assets: a writer with the byte layout of rosy_asset::asset::write
(src/Asset/Asset.cpp:28-407) and the Python side of the library's reader
(rz_rsy_* in include/rosy_gb300.h), which turns an asset into a renderable
Scene.

The writer exists so that assets can be produced on this side (the reference
builds them with its packager, src/Packager/Packager.cpp) and so that the
reader is tested against files with the reference's exact layout.
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass, field

import numpy as np

from . import _abi, _lib
from . import scene as sc

MAGIC = 0x52535946  # "RSYF"
VERSION = 1


@dataclass
class RsyNode:
    world_translate: tuple = (0.0, 0.0, 0.0)
    world_scale: float = 1.0
    world_yaw: float = 0.0
    transform: np.ndarray = field(default_factory=lambda: np.eye(4))  # (4, 4), row-major as a matrix
    mesh_id: int = 0xFFFFFFFF
    children: list = field(default_factory=list)
    name: str = ""


@dataclass
class RsyMesh:
    positions: np.ndarray  # (n, 16) float32, rosy_asset::position
    indices: np.ndarray    # (m,) uint32, mesh-local
    surfaces: list         # [(start_index, count, material, min_bounds(3), max_bounds(3))]


@dataclass
class RsyAsset:
    materials: np.ndarray                 # MATERIAL_DTYPE records (rz_material layout)
    samplers: np.ndarray                  # SAMPLER_DTYPE records
    scenes: list                          # [[node indices]]
    nodes: list                           # [RsyNode]
    images: list                          # [(image_type, name)]
    meshes: list                          # [RsyMesh]
    coordinate_system: np.ndarray = field(default_factory=lambda: np.eye(4))
    root_scene: int = 0


def _colmajor(m) -> list:
    return [float(v) for v in np.asarray(m, np.float64).T.reshape(-1)]


def write_rsy(path: str, a: RsyAsset) -> None:
    """Writes `a` in the .rsy layout: every count a little-endian u64 (size_t),
    materials as the 68-byte x64 record (u8 double_sided + 3 pad bytes, ...)."""
    out = bytearray()
    out += struct.pack("<III", MAGIC, VERSION, 1)
    out += struct.pack("<16f", *_colmajor(a.coordinate_system))
    out += struct.pack("<I", a.root_scene)
    out += struct.pack("<6Q", len(a.materials), len(a.samplers), len(a.scenes), len(a.nodes), len(a.images),
                       len(a.meshes))
    for m in a.materials:
        out += struct.pack("<B3x4fffB3xf8I", int(m["double_sided"]), *[float(v) for v in m["base_color_factor"]],
                           float(m["metallic_factor"]), float(m["roughness_factor"]), int(m["alpha_mode"]),
                           float(m["alpha_cutoff"]), int(m["color_image_index"]), int(m["color_sampler_index"]),
                           int(m["normal_image_index"]), int(m["normal_sampler_index"]),
                           int(m["metallic_image_index"]), int(m["metallic_sampler_index"]),
                           int(m["mixmap_image_index"]), int(m["mixmap_sampler_index"]))
    for s in a.samplers:
        out += struct.pack("<4H", int(s["min_filter"]), int(s["mag_filter"]), int(s["wrap_s"]), int(s["wrap_t"]))
    for nodes in a.scenes:
        out += struct.pack("<Q", len(nodes)) + struct.pack(f"<{len(nodes)}I", *nodes)
    for n in a.nodes:
        name = n.name.encode()
        out += struct.pack("<7Q", 1, 1, 1, 1, 1, len(n.children), len(name))
        out += struct.pack("<3f", *n.world_translate) + struct.pack("<ff", n.world_scale, n.world_yaw)
        out += struct.pack("<16f", *_colmajor(n.transform)) + struct.pack("<I", n.mesh_id)
        out += struct.pack(f"<{len(n.children)}I", *n.children) + name
    for t, name in a.images:
        nb = name.encode()
        out += struct.pack("<QQI", 1, len(nb), t) + nb
    for m in a.meshes:
        pos = np.ascontiguousarray(m.positions, np.float32).reshape(-1, 16)
        idx = np.ascontiguousarray(m.indices, np.uint32)
        out += struct.pack("<3Q", len(pos), len(idx), len(m.surfaces))
        out += pos.astype("<f4").tobytes() + idx.astype("<u4").tobytes()
        for start, count, mat, mn, mx in m.surfaces:
            out += struct.pack("<III3f3f", start, count, mat, *mn, *mx)
    with open(path, "wb") as f:
        f.write(bytes(out))


class RsyFile:
    """An .rsy file parsed by the library (rz_rsy_read)."""

    def __init__(self, path: str):
        self._lib = _lib.load()
        self._a = C.c_void_p()
        rc = self._lib.rz_rsy_read(path.encode(), C.byref(self._a))
        if rc != 0:
            raise _lib.RzError(rc, f"rz_rsy_read({path})")
        self.info = _abi.RzRsyInfo()
        self._check(self._lib.rz_rsy_get_info(self._a, C.byref(self.info)), "rz_rsy_get_info")

    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            raise _lib.RzError(rc, what)

    def close(self) -> None:
        if self._a:
            self._lib.rz_rsy_free(self._a)
            self._a = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def meshes(self) -> list[tuple[np.ndarray, np.ndarray]]:
        """[(positions (n, 16) float32, indices (m,) uint32)] copied out of the asset."""
        n = self.info.mesh_count
        arr = (_abi.RzMesh * max(n, 1))()
        self._check(self._lib.rz_rsy_get_meshes(self._a, arr, n), "rz_rsy_get_meshes")
        out = []
        for i in range(n):
            m = arr[i]
            pos = np.ctypeslib.as_array(C.cast(m.positions, C.POINTER(C.c_float)), (m.position_count * 16,)).copy() \
                if m.position_count else np.zeros(0, np.float32)
            idx = np.ctypeslib.as_array(C.cast(m.indices, C.POINTER(C.c_uint32)), (m.index_count,)).copy() \
                if m.index_count else np.zeros(0, np.uint32)
            out.append((pos.reshape(-1, 16), idx))
        return out

    def materials(self) -> np.ndarray:
        n = self.info.material_count
        out = np.zeros(n, sc.MATERIAL_DTYPE)
        self._check(self._lib.rz_rsy_get_materials(self._a, _abi.ptr(out), n), "rz_rsy_get_materials")
        return out

    def samplers(self) -> np.ndarray:
        n = self.info.sampler_count
        out = np.zeros(n, sc.SAMPLER_DTYPE)
        self._check(self._lib.rz_rsy_get_samplers(self._a, _abi.ptr(out), n), "rz_rsy_get_samplers")
        return out

    def images(self) -> list[tuple[int, str]]:
        res = []
        for i in range(self.info.image_count):
            t = C.c_uint32()
            ln = C.c_uint32()
            self._check(self._lib.rz_rsy_get_image(self._a, i, C.byref(t), None, 0, C.byref(ln)), "rz_rsy_get_image")
            buf = C.create_string_buffer(ln.value + 1)
            self._check(self._lib.rz_rsy_get_image(self._a, i, None, buf, ln.value + 1, None), "rz_rsy_get_image")
            res.append((t.value, buf.value.decode(errors="replace")))
        return res

    def scene_objects(self) -> tuple[np.ndarray, np.ndarray]:
        """(objects (k, 41) float32, surfaces SURFACE_DTYPE) of the flattened root scene."""
        objs = np.zeros((self.info.object_count, sc.OBJECT_FLOATS), np.float32)
        surfs = np.zeros(self.info.surface_count, sc.SURFACE_DTYPE)
        self._check(self._lib.rz_rsy_get_scene(self._a, _abi.ptr(objs), len(objs), _abi.ptr(surfs), len(surfs)),
                    "rz_rsy_get_scene")
        return objs, surfs


def _load_images(path: str, imgs: list[tuple[int, str]]) -> tuple[list, list[str]]:
    """One texture per asset image: the named .dds file read as BC7 (the name as
    given, else relative to the .rsy file's folder), or, where no such file can
    be read, a 1x1 white texture of the image's type — the engine warns and
    skips an unreadable image (src/Engine/Graphics.cpp:3609-3613)."""
    import os

    from .dds import texture_from_dds

    out, missing = [], []
    base = os.path.dirname(os.path.abspath(path))
    for kind, name in imgs:
        tex = None
        for cand in (name, os.path.join(base, name)):
            if name and os.path.isfile(cand):
                try:
                    tex = texture_from_dds(cand, kind)
                    break
                except _lib.RzError:
                    pass
        if tex is None:
            missing.append(name)
            tex = sc.Texture(1, 1, 1, kind, np.full(4, 255, np.uint8))
        out.append(tex)
    return out, missing


def scene_from_rsy(path: str, textures: list | None = None, width: int = 640, height: int = 360,
                   shadow_size: int = 1024, camera_position=(0.0, 0.0, 3.0), sun_direction=(0.3, 1.0, 0.2)) -> sc.Scene:
    """A renderable Scene from an .rsy file. The asset's images are named .dds
    files; without `textures` (one scene.Texture per image) they are read as BC7
    textures (decoded on the device when the scene is uploaded), and an image
    whose file is missing becomes a 1x1 white texture of its type (the scene's
    `missing_images` lists them). Camera and light are the given ones (the level
    supplies them in the engine)."""
    f = RsyFile(path)
    try:
        meshes = f.meshes()
        mats = f.materials()
        smps = f.samplers()
        imgs = f.images()
        objs, surfs = f.scene_objects()
    finally:
        f.close()
    verts = np.concatenate([m[0] for m in meshes]).astype(np.float32) if meshes else np.zeros((0, 16), np.float32)
    idx = np.concatenate([m[1] for m in meshes]).astype(np.uint32) if meshes else np.zeros(0, np.uint32)
    table, vo, io = [], 0, 0
    for p, i in meshes:
        table.append((vo, len(p), io, len(i)))
        vo += len(p)
        io += len(i)
    missing: list[str] = []
    if textures is None:
        textures, missing = _load_images(path, imgs)
    sun_position, spn = sc.sun_matrices(np.asarray(sun_direction, np.float64))
    view = sc.camera_look_at_origin(camera_position)
    import math

    rec = sc.scene_record(view, sc.projection(width / height, math.radians(60.0)), sun_position, spn,
                          np.asarray(camera_position, np.float64), width, height)
    out = sc.Scene(name=f"rsy:{path}", width=width, height=height, shadow_size=shadow_size, vertices=verts,
                   indices=idx, meshes=table, objects=objs, surfaces=surfs, materials=mats, textures=list(textures),
                   samplers=smps if len(smps) else sc.linear_sampler(), scene=rec,
                   draw_config=sc.default_draw_config(), cameras=[rec])
    out.missing_images = missing
    return out
