"""The shadow depth entry point that allocates nothing (rz_shadow_depth_static).

Callers that cannot allocate device memory while running (engines with their
own allocator or a fixed memory budget, frame loops that must not call
cudaMalloc/cudaFree) use this entry point; its scratch is a fixed array
compiled into the library, shared by every call. The tests check its depth
maps against the oracle and against rz_render's shadow pass, that one call's
leftovers in the shared array never reach the next call (a large draw and then
a smaller one on a smaller target, calls after each kind of overflow), that
both overflow causes are reported, and that device memory stays the same
across a call. This file is collected last so that a failure here comes after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from rosy_gb300 import _lib
from rosy_gb300 import scene as sc
from rosy_gb300.graphics import render_scene

RZ_OK, RZ_INVALID_ARGUMENT, RZ_OVERFLOW = 0, 3, 14

pytestmark = pytest.mark.gpu


def _clip_scene(pos, size, cull=False):
    """One draw of the clip-space triangles `pos` (n*3, 3) with identity world and
    shadow projection, for the oracle's shadow pass on a size x size map."""
    n = len(pos)
    verts = np.zeros((n, sc.VERTEX_FLOATS), np.float32)
    verts[:, 0:3] = pos
    verts[:, 3:6] = (0, 0, 1)
    verts[:, 6:10] = (1, 0, 0, 1)
    verts[:, 10:14] = 1.0
    eye = np.eye(4)
    rec = sc.scene_record(eye, eye, (0, 0, 10, 1), eye, (0, 0, 5), 8, 8)
    rec["shadow_projection_near"] = sc.colmajor(eye)
    dc = sc.default_draw_config()
    dc["cull_enabled"] = 1 if cull else 0
    dc["depth_bias_enabled"] = 0
    surf = np.zeros(1, sc.SURFACE_DTYPE)
    surf["index_count"] = n
    surf["material_index"] = sc.U32_MAX
    return sc.Scene(name="clip", width=8, height=8, shadow_size=size, vertices=verts,
                    indices=np.arange(n, dtype=np.uint32), meshes=[(0, n, 0, n)],
                    objects=sc.object_record(eye)[None, :], surfaces=surf,
                    materials=np.zeros(0, sc.MATERIAL_DTYPE), textures=[], samplers=sc.linear_sampler(),
                    scene=rec, draw_config=dc, cameras=[rec])


def _lit_scene(seed, triangles, size):
    """Random triangles under a light that sees the whole mesh large in the map."""
    s = sc.random_triangles(seed=seed, triangles=triangles, width=64, height=48, shadow_size=size, texture_size=16)
    s.scene["shadow_projection_near"] = sc.colmajor(
        np.diag([0.9, 0.9, -0.2, 1.0]) @ np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, -3.0], [0, 0, 0, 1.0]]))
    s.cameras = [s.scene]
    return s


def _small_triangles(count, size, px=24.0, seed=0):
    """`count` clip-space triangles of up to about `px` pixels on a side on a
    size x size map, both windings, at depths in (0.05, 0.95)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(-1.0, 1.0, (count, 1, 2))
    d = rng.uniform(-1.0, 1.0, (count, 3, 2)) * (px / size)
    tris = np.zeros((count, 3, 3), np.float32)
    tris[:, :, :2] = c + d
    tris[:, :, 2] = rng.uniform(0.05, 0.95, (count, 3))
    return tris.reshape(-1, 3)


def _call(lib, s, depth, stream=None):
    """rz_shadow_depth_static on the scene's single draw, into `depth` (size^2 f32)."""
    import torch

    pos = np.zeros((len(s.vertices), 4), np.float32)
    pos[:, :3] = s.vertices[:, 0:3]
    d_pos = torch.from_numpy(pos).cuda()
    d_idx = torch.from_numpy(s.indices.astype(np.int64)).to(torch.int32).cuda()
    proj = (C.c_float * 16)(*s.scene["shadow_projection_near"][0].tolist())
    world = (C.c_float * 16)(*s.objects[0, 0:16].tolist())
    dc = np.ascontiguousarray(s.draw_config)
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    rc = lib.rz_shadow_depth_static(d_pos.data_ptr(), len(pos), d_idx.data_ptr(), len(s.indices), proj, world,
                                    dc.ctypes.data, s.shadow_size, s.shadow_size, depth.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc


def _depth(size, fill=0.5):
    import torch

    return torch.full((size, size), fill, dtype=torch.float32, device="cuda")


def _bits(t):
    return t.cpu().numpy().view(np.uint32)


def test_static_shadow_pass_matches_oracle_and_render_twice(gpu, oracle):
    """Two calls in a row through the C ABI equal the oracle's shadow map and
    rz_render's, bit for bit."""
    s = _lit_scene(11, 600, 256)
    ref = oracle.raster(s)["shadow"]
    assert (ref > 0).mean() > 0.05
    assert np.array_equal(render_scene(s)["shadow"].view(np.uint32), ref.view(np.uint32))
    lib = _lib.load()
    for _ in range(2):
        depth = _depth(s.shadow_size)
        assert _call(lib, s, depth) == RZ_OK
        assert np.array_equal(_bits(depth), ref.view(np.uint32))


def test_large_draw_then_smaller_draw_on_smaller_target(gpu, oracle):
    """A draw with many records on a 1024^2 map, then a small draw on a 200^2
    map (with culling), then both again: each equals the oracle, so nothing the
    previous call left in the shared array (records, chunk map, header) leaks in."""
    lib = _lib.load()
    big = _clip_scene(_small_triangles(16000, 1024, px=40.0, seed=1), 1024)
    small = _clip_scene(_small_triangles(700, 200, px=30.0, seed=2), 200, cull=True)
    for s in (big, small, big, small):
        depth = _depth(s.shadow_size)
        assert _call(lib, s, depth) == RZ_OK
        ref = oracle.raster(s)["shadow"]
        assert (ref > 0).mean() > 0.05
        assert np.array_equal(_bits(depth), ref.view(np.uint32))


def _full_target_triangles(count):
    """`count` triangles that each cover the whole target, at rising depths."""
    tris = []
    for i in range(count):
        z = 0.1 + 0.8 * i / max(count, 1)
        tris += [(-1.0, -1.0, z), (3.0, -1.0, z), (-1.0, 3.0, z)]
    return np.asarray(tris, np.float32)


def _fanning_triangles(count, size, seed=0):
    """`count` triangles of about 25 pixels on a side that cross both the z = 0
    and the z = w planes, so that clipping cuts each into a pentagon (three
    setup records each)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = 50.0 / size
    c = rng.uniform(-0.9, 0.9 - d, (count, 2))
    tris = np.zeros((count, 3, 3), np.float32)
    tris[:, 0, :2] = c
    tris[:, 1, :2] = c + (d, 0.0)
    tris[:, 2, :2] = c + (0.0, d)
    tris[:, :, 2] = (-0.5, 1.5, 0.5)
    return tris.reshape(-1, 3)


def test_chunk_overflow_then_normal_call(gpu, oracle):
    """Eight triangles covering a whole 4096^2 map need 8 x 16,384 chunks of 32
    stamps, more than the fixed 65,536: RZ_OVERFLOW. The next call is exact."""
    lib = _lib.load()
    over = _clip_scene(_full_target_triangles(8), 4096)
    assert _call(lib, over, _depth(4096)) == RZ_OVERFLOW
    s = _lit_scene(31, 900, 320)
    depth = _depth(s.shadow_size)
    assert _call(lib, s, depth) == RZ_OK
    assert np.array_equal(_bits(depth), oracle.raster(s)["shadow"].view(np.uint32))


def test_record_overflow_from_clipping_then_normal_call(gpu, oracle):
    """16,384 triangles that clipping fans out into about 49,000 records, twice
    the fixed record space: RZ_OVERFLOW (not a chunk overflow: their stamps fill
    about half the chunk queue). A draw of the same triangles that fits is
    exact, and so is the next ordinary call."""
    lib = _lib.load()
    size = 1024
    tris = _fanning_triangles(16384, size)
    over = _clip_scene(tris, size)
    assert _call(lib, over, _depth(size)) == RZ_OVERFLOW
    fits = _clip_scene(tris[: 3 * 4000], size)
    depth = _depth(size)
    assert _call(lib, fits, depth) == RZ_OK
    ref = oracle.raster(fits)["shadow"]
    assert (ref > 0).mean() > 0.1
    assert np.array_equal(_bits(depth), ref.view(np.uint32))
    s = _lit_scene(41, 800, 256)
    depth = _depth(s.shadow_size)
    assert _call(lib, s, depth) == RZ_OK
    assert np.array_equal(_bits(depth), oracle.raster(s)["shadow"].view(np.uint32))


def test_static_shadow_pass_leaves_device_memory_unchanged(gpu):
    """After a warm-up call, a call changes the device's free memory by nothing."""
    import torch

    lib = _lib.load()
    s = _clip_scene(_small_triangles(3000, 512, seed=3), 512)
    pos = np.zeros((len(s.vertices), 4), np.float32)
    pos[:, :3] = s.vertices[:, 0:3]
    d_pos = torch.from_numpy(pos).cuda()
    d_idx = torch.from_numpy(s.indices.astype(np.int64)).to(torch.int32).cuda()
    depth = _depth(s.shadow_size)
    proj = (C.c_float * 16)(*s.scene["shadow_projection_near"][0].tolist())
    world = (C.c_float * 16)(*s.objects[0, 0:16].tolist())
    dc = np.ascontiguousarray(s.draw_config)
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        return lib.rz_shadow_depth_static(d_pos.data_ptr(), len(pos), d_idx.data_ptr(), len(s.indices), proj, world,
                                          dc.ctypes.data, s.shadow_size, s.shadow_size, depth.data_ptr(), stream)

    torch.cuda.synchronize()
    assert call() == RZ_OK
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert call() == RZ_OK
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_static_shadow_pass_rejects_oversized_draws(gpu):
    import torch

    lib = _lib.load()
    depth = torch.zeros(16, dtype=torch.float32, device="cuda")
    pos = torch.zeros((4, 4), dtype=torch.float32, device="cuda")
    idx = torch.zeros(3 * 16385, dtype=torch.int32, device="cuda")
    eye = (C.c_float * 16)(*np.eye(4, dtype=np.float32).reshape(-1).tolist())
    dc = np.ascontiguousarray(sc.default_draw_config())
    rc = lib.rz_shadow_depth_static(pos.data_ptr(), 4, idx.data_ptr(), 3 * 16385, eye, eye, dc.ctypes.data, 4, 4,
                                    depth.data_ptr(), None)
    assert rc == RZ_INVALID_ARGUMENT
