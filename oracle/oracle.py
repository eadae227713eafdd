"""ORACLE — test infrastructure only (tests, smoke check, CPU baseline of the
bench). ctypes binding of the scalar C++ restatement in rz_oracle.cpp.

Parity is unpinned by the reference: Rosy has no tests or golden data and cannot
run here; hand-derived known-answer tests pin the restatement instead. The BC7
decoder (bc7_oracle.cpp) is pinned against the GPU texture unit's own BC7
decoding, the decoder behind the reference's images (tests/golden/bc7_hw.npz).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from rosy_gb300._abi import Marshalled, ptr  # noqa: E402

BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "librz_oracle.so")
SOURCES = [os.path.join(HERE, "rz_oracle.cpp"), os.path.join(HERE, "bc7_oracle.cpp")]


def build(force: bool = False) -> str:
    """Compiles the oracle with g++ (portable flags, no FMA contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    deps = SOURCES + [os.path.join(HERE, "oracle.h"), os.path.join(ROOT, "include", "rosy_gb300.h")]
    if not force and os.path.exists(LIB_PATH):
        mt = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= mt for d in deps):
            return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-Wall", "-o", tmp] + SOURCES
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class OracleScene(C.Structure):
    _fields_ = [
        ("vertices", C.c_void_p), ("vertex_count", C.c_uint32), ("index_count", C.c_uint32),
        ("indices", C.c_void_p), ("meshes", C.c_void_p), ("mesh_count", C.c_uint32),
        ("object_count", C.c_uint32), ("objects", C.c_void_p), ("surfaces", C.c_void_p),
        ("surface_count", C.c_uint32), ("material_count", C.c_uint32), ("materials", C.c_void_p),
        ("textures", C.c_void_p), ("texture_count", C.c_uint32), ("sampler_count", C.c_uint32),
        ("samplers", C.c_void_p), ("scene", C.c_void_p), ("draw_config", C.c_void_p),
        ("width", C.c_uint32), ("height", C.c_uint32), ("shadow_size", C.c_uint32),
        ("samples", C.c_uint32), ("debug_object_count", C.c_uint32), ("debug_objects", C.c_void_p),
    ]


class OracleOut(C.Structure):
    _fields_ = [("color", C.c_void_p), ("depth", C.c_void_p), ("ids", C.c_void_p),
                ("shadow", C.c_void_p), ("color_f64", C.c_void_p), ("texel_bytes", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        for fn in (_lib.oracle_render, _lib.oracle_raster):
            fn.argtypes = [C.POINTER(OracleScene), C.POINTER(OracleOut), C.c_int]
            fn.restype = C.c_int
        _lib.oracle_bc7_decode.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
        _lib.oracle_bc7_decode.restype = C.c_int
        _lib.oracle_subpixel_sources.argtypes = [C.POINTER(OracleScene), C.c_void_p, C.c_void_p, C.c_int]
        _lib.oracle_subpixel_sources.restype = C.c_int
    return _lib


def _scene_struct(m: Marshalled) -> OracleScene:
    s = m.scene
    o = OracleScene()
    o.vertices = ptr(m.vertices)
    o.vertex_count = len(m.vertices)
    o.indices = ptr(m.indices)
    o.index_count = len(m.indices)
    o.meshes = ptr(m.mesh_table)
    o.mesh_count = len(m.mesh_table)
    o.objects = ptr(m.objects)
    o.object_count = len(m.objects)
    o.surfaces = ptr(m.surfaces)
    o.surface_count = len(m.surfaces)
    o.materials = ptr(m.materials)
    o.material_count = len(m.materials)
    o.textures = C.cast(m.textures, C.c_void_p)
    o.texture_count = m.n_textures
    o.samplers = ptr(m.samplers)
    o.sampler_count = len(m.samplers)
    o.scene = ptr(m.scene_rec)
    o.draw_config = ptr(m.draw_config)
    o.width, o.height, o.shadow_size = s.width, s.height, s.shadow_size
    o.samples = getattr(s, "samples", 1)
    if m.debug_objects is not None and len(m.debug_objects):
        o.debug_objects = ptr(m.debug_objects)
        o.debug_object_count = len(m.debug_objects)
    return o


def cascades(s) -> int:
    """Shadow cascades of the scene's draw config (1..4)."""
    n = int(s.draw_config["shadow_cascades"][0]) if "shadow_cascades" in s.draw_config.dtype.names else 1
    return min(max(n, 1), 4)


def _shadow_array(s) -> np.ndarray:
    """(S, S) for one shadow map, (cascades, S, S) for several."""
    n = cascades(s)
    shape = (s.shadow_size, s.shadow_size) if n == 1 else (n, s.shadow_size, s.shadow_size)
    return np.zeros(shape, np.float32)


def _sample_shape(s) -> tuple:
    """(H, W) with one sample per pixel, (4, H, W) with 4x multisampling."""
    return (s.height, s.width) if getattr(s, "samples", 1) != 4 else (4, s.height, s.width)


def render(s, threads: int = 0, fp64: bool = False, texel_bytes: bool = False) -> dict:
    """Full frame: colour (H,W,4) u8 (resolved), depth and ids per sample ((H,W), or (4,H,W)
    with 4x multisampling), shadow (S,S) f32 (or (cascades,S,S)), optionally color_f64
    (H,W,4) and the compulsory texel bytes of the shading."""
    m = Marshalled(s)
    o = _scene_struct(m)
    out = {
        "color": np.zeros((s.height, s.width, 4), np.uint8),
        "depth": np.zeros(_sample_shape(s), np.float32),
        "ids": np.zeros(_sample_shape(s), np.uint32),
        "shadow": _shadow_array(s),
    }
    oo = OracleOut(ptr(out["color"]), ptr(out["depth"]), ptr(out["ids"]), ptr(out["shadow"]), None, None)
    if fp64:
        out["color_f64"] = np.zeros((s.height, s.width, 4), np.float64)
        oo.color_f64 = ptr(out["color_f64"])
    tb = np.zeros(1, np.uint64)
    if texel_bytes:
        oo.texel_bytes = ptr(tb)
    rc = lib().oracle_render(C.byref(o), C.byref(oo), int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_render failed: {rc}")
    if texel_bytes:
        out["texel_bytes"] = int(tb[0])
    return out


def raster(s, threads: int = 0) -> dict:
    """Raster passes only: depth, ids, shadow."""
    m = Marshalled(s)
    o = _scene_struct(m)
    out = {
        "depth": np.zeros(_sample_shape(s), np.float32),
        "ids": np.zeros(_sample_shape(s), np.uint32),
        "shadow": _shadow_array(s),
    }
    oo = OracleOut(None, ptr(out["depth"]), ptr(out["ids"]), ptr(out["shadow"]), None, None)
    rc = lib().oracle_raster(C.byref(o), C.byref(oo), int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_raster failed: {rc}")
    return out


def subpixel_sources(s, ids: np.ndarray, threads: int = 0) -> np.ndarray:
    """(H, W) u16 sub-pixel source masks of the learned path's x2 base for the
    scene's camera and the (H, W) visibility `ids` (triangle id + 1)."""
    m = Marshalled(s)
    o = _scene_struct(m)
    ids = np.ascontiguousarray(ids, np.uint32).reshape(s.height, s.width)
    out = np.zeros((s.height, s.width), np.uint16)
    rc = lib().oracle_subpixel_sources(C.byref(o), ptr(ids), ptr(out), int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_subpixel_sources failed: {rc}")
    return out


def bc7_decode(blocks: np.ndarray, width: int, height: int) -> np.ndarray:
    """One image of BC7 blocks (bytes, max(1,(w+3)/4) x max(1,(h+3)/4) blocks in
    rows) decoded to (height, width, 4) RGBA8 by the scalar restatement."""
    b = np.ascontiguousarray(blocks, np.uint8).reshape(-1)
    need = max(1, (width + 3) // 4) * max(1, (height + 3) // 4) * 16
    assert b.size >= need, (b.size, need)
    out = np.zeros((height, width, 4), np.uint8)
    rc = lib().oracle_bc7_decode(ptr(b), width, height, ptr(out))
    assert rc == 0, rc
    return out
