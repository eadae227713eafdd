"""Python host mirror of Rosy's renderer interface over the C ABI.

``Graphics`` follows ``rosy::graphics`` (src/Engine/Graphics.h:11-21):
init / update / render / resize / deinit, every call returning or raising on a
``rosy::result`` code, plus the inner seams the engine drives through
``graphics::update`` (set_asset, set_graphic_objects, the mob transform update;
src/Engine/Graphics.cpp:6172-6197). Rendering is headless: the frame stays in
device memory, readable as device pointers or copied to host arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi, _lib
from . import scene as sc
from .scene import Scene


class Graphics:
    def __init__(self):
        self._ctx = C.c_void_p()
        self._lib = None
        self._marshalled = None
        self.viewport_width = 0
        self.viewport_height = 0
        self.shadow_size = 0

    # -- rosy::graphics -----------------------------------------------------------
    def init(self, width: int, height: int, shadow_size: int = 4096, device: int = 0, queue_chunks: int = 0,
             samples: int = 1) -> None:
        """graphics::init: creates the context (stream + frame buffers) on `device`; samples = 4
        renders the camera pass with the reference's 4x multisampling."""
        self._lib = _lib.load()
        cfg = _abi.RzConfig(width=width, height=height, shadow_map_size=shadow_size, samples=samples, device=device,
                            queue_chunks=queue_chunks)
        self.samples = samples
        rc = self._lib.rz_create(C.byref(self._ctx), C.byref(cfg))
        if rc != 0:
            raise _lib.RzError(rc, "rz_create")
        self.viewport_width, self.viewport_height, self.shadow_size = width, height, shadow_size

    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            raise _lib.RzError(rc, what, self._lib.rz_last_error(self._ctx).decode(errors="replace"))

    def set_asset(self, scene: Scene) -> None:
        """graphics_device::set_asset: meshes, materials, textures, samplers."""
        m = _abi.Marshalled(scene)
        self._marshalled = m
        self._check(self._lib.rz_set_asset(
            self._ctx, C.cast(m.meshes, C.c_void_p), len(scene.meshes),
            _abi.ptr(m.materials), len(m.materials),
            C.cast(m.textures, C.c_void_p), m.n_textures,
            _abi.ptr(m.samplers), len(m.samplers)), "rz_set_asset")

    def set_graphic_objects(self, objects: np.ndarray, surfaces: np.ndarray) -> None:
        """graphics_device::set_graphic_objects: transforms + surface list in scene order."""
        objects = np.ascontiguousarray(objects, np.float32)
        surfaces = np.ascontiguousarray(surfaces)
        self._check(self._lib.rz_set_objects(self._ctx, _abi.ptr(objects), len(objects),
                                             _abi.ptr(surfaces), len(surfaces)), "rz_set_objects")

    # -- batched views -------------------------------------------------------------
    def add_scene(self, scene: Scene) -> int:
        """Appends a scene (asset + objects + surfaces); returns its index."""
        m = _abi.Marshalled(scene)
        self._batch_keep = getattr(self, "_batch_keep", []) + [m]
        idx = C.c_uint32()
        self._check(self._lib.rz_add_scene(
            self._ctx, C.cast(m.meshes, C.c_void_p), len(scene.meshes), _abi.ptr(m.materials), len(m.materials),
            C.cast(m.textures, C.c_void_p), m.n_textures, _abi.ptr(m.samplers), len(m.samplers),
            _abi.ptr(m.objects), len(m.objects), _abi.ptr(m.surfaces), len(m.surfaces), C.byref(idx)), "rz_add_scene")
        return int(idx.value)

    def set_views(self, views) -> None:
        """views: sequence of (scene_index, width, height, shadow_map_size, draw_config record)."""
        arr = (_abi.RzView * len(views))()
        for i, (sc_i, w, h, sz, dc) in enumerate(views):
            arr[i].scene, arr[i].width, arr[i].height, arr[i].shadow_map_size = sc_i, w, h, sz
            C.memmove(C.byref(arr[i].draw_config), np.ascontiguousarray(dc).ctypes.data, 32)
        self._views = list(views)
        self._check(self._lib.rz_set_views(self._ctx, arr, len(views)), "rz_set_views")

    def set_tuning(self, chunk_stamps: int = 32, small_extent: int = 8, queue_chunks: int = 0,
                   batched: bool = True) -> None:
        t = _abi.RzTuning(chunk_stamps, small_extent, queue_chunks, 1 if batched else 0)
        self._check(self._lib.rz_set_tuning(self._ctx, C.byref(t)), "rz_set_tuning")

    def set_wait_limit(self, lookback_spins: int) -> None:
        """Bound of each look-back wait of the blended list's ordered setup (0: default)."""
        self._check(self._lib.rz_set_wait_limit(self._ctx, lookback_spins), "rz_set_wait_limit")

    def tuning(self) -> dict:
        t = _abi.RzTuning()
        self._check(self._lib.rz_get_tuning(self._ctx, C.byref(t)), "rz_get_tuning")
        return {"chunk_stamps": t.chunk_stamps, "small_extent": t.small_extent, "queue_chunks": t.queue_chunks,
                "batched": bool(t.batched)}

    def autotune(self, frames: int = 5) -> tuple[dict, list]:
        """Tries chunk_stamps in {16,32,64} x small_extent in {4,8,12}; applies the fastest."""
        t = _abi.RzTuning()
        ms = (C.c_float * 9)()
        self._check(self._lib.rz_autotune(self._ctx, frames, C.byref(t), ms, 9), "rz_autotune")
        return self.tuning(), [float(x) for x in ms]

    def update_view(self, view: int, scene_data: np.ndarray) -> None:
        sd = np.ascontiguousarray(scene_data)
        self._check(self._lib.rz_update_view(self._ctx, view, _abi.ptr(sd)), "rz_update_view")

    def download_view(self, view: int) -> dict:
        """Colour, depth, ids and shadow map of one view of the last frame."""
        f = _abi.RzFrameOut()
        self._check(self._lib.rz_get_view_frame(self._ctx, view, C.byref(f)), "rz_get_view_frame")
        self.sync()
        W, H, S = f.width, f.height, f.shadow_map_size
        v = getattr(self, "_views", None)
        n = min(max(int(v[view][4]["shadow_cascades"][0]), 1), 4) if v else 1
        ns = getattr(self, "samples", 1)
        out = {
            "vis": device_array(f.visibility_u64, (H, W) if ns == 1 else (ns, H, W), np.uint64),
            "shadow": device_array(f.shadow_map_f32, (S, S) if n == 1 else (n, S, S), np.float32),
            "color": device_array(f.color_rgba8, (H, W, 4), np.uint8),
            "depth": device_array(f.depth_f32, (H, W), np.float32),
        }
        ids = (out["vis"] & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        out["ids"] = np.where(ids > 0, ids - np.uint32(f.triangle_id_base), 0).astype(np.uint32)
        out["vis_depth"] = (out["vis"] >> np.uint64(32)).astype(np.uint32).view(np.float32)
        return out

    def set_gbuffer(self, enable: bool) -> None:
        """Makes the shading pass also write albedo and octahedral normals (the upsampler's inputs)."""
        self._check(self._lib.rz_set_gbuffer(self._ctx, 1 if enable else 0), "rz_set_gbuffer")

    def set_debug_objects(self, objects: np.ndarray | None) -> None:
        """The debug-line overlay of every following frame (DEBUG_OBJECT_DTYPE records, drawn in
        order after the blended list); None or an empty array turns it off."""
        if objects is None or len(objects) == 0:
            self._check(self._lib.rz_set_debug_objects(self._ctx, None, 0), "rz_set_debug_objects")
            return
        objs = np.ascontiguousarray(objects, sc.DEBUG_OBJECT_DTYPE)
        self._check(self._lib.rz_set_debug_objects(self._ctx, _abi.ptr(objs), len(objs)), "rz_set_debug_objects")

    def gbuffer(self, view: int = 0) -> _abi.RzGbuffer:
        """Device pointers of one view's G-buffer (after sync)."""
        g = _abi.RzGbuffer()
        self._check(self._lib.rz_get_view_gbuffer(self._ctx, view, C.byref(g)), "rz_get_view_gbuffer")
        return g

    def download_gbuffer(self, view: int = 0) -> dict:
        """Host copies of one view's G-buffer: colour and albedo (H, W, 4) u8, depth (H, W) f32,
        normal (H, W, 2) f16, and (single-sampled frames) the sub-pixel sources (H, W) u16."""
        self.sync()
        g = self.gbuffer(view)
        H, W = g.height, g.width
        out = {
            "color": device_array(g.color_rgba8, (H, W, 4), np.uint8),
            "depth": device_array(g.depth_f32, (H, W), np.float32),
            "albedo": device_array(g.albedo_rgba8, (H, W, 4), np.uint8),
            "normal": device_array(g.normal_oct_f16x2, (H, W, 2), np.float16),
        }
        if g.sources_u16:
            out["sources"] = device_array(g.sources_u16, (H, W), np.uint16)
        return out

    def update_objects(self, offset: int, objects: np.ndarray) -> None:
        """The go_update upload (mob transforms) of src/Engine/Graphics.cpp:5120-5138."""
        objects = np.ascontiguousarray(objects, np.float32)
        self._check(self._lib.rz_update_objects(self._ctx, offset, _abi.ptr(objects), len(objects)),
                    "rz_update_objects")

    def set_draw_config(self, draw_config: np.ndarray) -> None:
        dc = np.ascontiguousarray(draw_config)
        self._cascades = min(max(int(dc["shadow_cascades"][0]), 1), 4)
        self._check(self._lib.rz_set_draw_config(self._ctx, _abi.ptr(dc)), "rz_set_draw_config")

    def update(self, scene_data: np.ndarray) -> None:
        """graphics::update: the scene constants (gpu_scene_data) of the next frame."""
        sd = np.ascontiguousarray(scene_data)
        assert sd.nbytes == 408
        self._check(self._lib.rz_update(self._ctx, _abi.ptr(sd)), "rz_update")

    def render(self) -> None:
        """graphics::render: enqueue the frame on the context's stream."""
        self._check(self._lib.rz_render(self._ctx), "rz_render")

    def resize(self, width: int, height: int) -> None:
        self._check(self._lib.rz_resize(self._ctx, width, height), "rz_resize")
        self.viewport_width, self.viewport_height = width, height

    def deinit(self) -> None:
        if self._lib is not None and self._ctx:
            self._lib.rz_destroy(self._ctx)
        self._ctx = C.c_void_p()

    # -- headless outputs -------------------------------------------------------------
    def sync(self, timeout_ms: int = 0) -> None:
        self._check(self._lib.rz_sync(self._ctx, timeout_ms), "rz_sync")

    def sync_code(self, timeout_ms: int = 0) -> int:
        return int(self._lib.rz_sync(self._ctx, timeout_ms))

    def frame(self) -> _abi.RzFrameOut:
        out = _abi.RzFrameOut()
        self._check(self._lib.rz_get_frame(self._ctx, C.byref(out)), "rz_get_frame")
        return out

    def read_sync(self, pending: int = 0, timeout_ms: int = 0) -> None:
        """Waits until at most `pending` (0 or 1) read-backs are still travelling."""
        self._check(self._lib.rz_read_sync(self._ctx, pending, timeout_ms), "rz_read_sync")

    def read_frame(self, color: np.ndarray | None = None, depth: np.ndarray | None = None) -> None:
        """Enqueues device-to-host copies into caller arrays (complete after sync() or read_sync())."""
        cp = _abi.ptr(color) if color is not None else None
        dp = _abi.ptr(depth) if depth is not None else None
        self._check(self._lib.rz_read_frame(self._ctx, cp, color.nbytes if color is not None else 0,
                                            dp, depth.nbytes if depth is not None else 0), "rz_read_frame")

    def stats(self) -> _abi.RzStats:
        s = _abi.RzStats()
        self._check(self._lib.rz_get_stats(self._ctx, C.byref(s)), "rz_get_stats")
        return s

    STAGES = ("shadow_clear", "shadow_setup", "shadow_raster", "camera_clear", "camera_setup",
              "camera_raster", "shade")

    def set_stage_timing(self, enable: bool) -> None:
        self._check(self._lib.rz_set_stage_timing(self._ctx, 1 if enable else 0), "rz_set_stage_timing")

    def stage_times(self) -> dict:
        """Milliseconds per stage of the last completed frame (stage timing must be on)."""
        buf = (C.c_float * 16)()
        n = C.c_uint32()
        self._check(self._lib.rz_get_stage_times(self._ctx, buf, 16, C.byref(n)), "rz_get_stage_times")
        return {self.STAGES[i]: float(buf[i]) for i in range(n.value)}

    @property
    def stream(self) -> int:
        return int(self._lib.rz_get_stream(self._ctx) or 0)

    def download(self) -> dict:
        """Colour (H,W,4) u8, depth (H,W) f32, ids (H,W) u32 and shadow (S,S) f32 of the last frame."""
        f = self.frame()
        W, H, S = self.viewport_width, self.viewport_height, self.shadow_size
        self.sync()
        n = getattr(self, "_cascades", 1)
        ns = getattr(self, "samples", 1)
        out = {
            "vis": device_array(f.visibility_u64, (H, W) if ns == 1 else (ns, H, W), np.uint64),
            "shadow": device_array(f.shadow_map_f32, (S, S) if n == 1 else (n, S, S), np.float32),
        }
        color = np.empty((H, W, 4), np.uint8)
        depth = np.empty((H, W), np.float32)
        self.read_frame(color, depth)
        self.sync()
        out["color"] = color
        out["depth"] = depth
        out["ids"] = (out["vis"] & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        out["vis_depth"] = (out["vis"] >> np.uint64(32)).astype(np.uint32).view(np.float32)
        return out


class _DeviceView:
    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def device_array(ptr: int, shape, dtype) -> np.ndarray:
    """Copies a device buffer of the renderer to a host numpy array (torch as plumbing)."""
    import torch

    dt = np.dtype(dtype)
    if dt == np.uint64:  # torch has no uint64 copy path on every version: move raw int64
        view = torch.as_tensor(_DeviceView(ptr, shape, "<i8"), device="cuda")
        return view.cpu().numpy().view(np.uint64)
    if dt == np.uint16:  # nor a uint16 one: move raw int16
        view = torch.as_tensor(_DeviceView(ptr, shape, "<i2"), device="cuda")
        return view.cpu().numpy().view(np.uint16)
    view = torch.as_tensor(_DeviceView(ptr, shape, dt.str), device="cuda")
    return view.cpu().numpy()


def render_scene(scene: Scene, device: int = 0) -> dict:
    """Convenience: one frame of `scene` through the C ABI, downloaded to host arrays."""
    g = Graphics()
    g.init(scene.width, scene.height, scene.shadow_size, device, samples=getattr(scene, "samples", 1))
    try:
        g.set_asset(scene)
        g.set_graphic_objects(scene.objects, scene.surfaces)
        g.set_draw_config(scene.draw_config)
        if getattr(scene, "debug_objects", None) is not None:
            g.set_debug_objects(scene.debug_objects)
        g.update(scene.scene)
        g.render()
        if g.sync_code() == 14:  # RZ_OVERFLOW: the work queue grew; render the frame again
            g.render()
        g.sync()
        return g.download()
    finally:
        g.deinit()
