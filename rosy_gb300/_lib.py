"""Loads the in-tree renderer library and declares the C ABI signatures.

There is no fallback: if the library has not been built, or the process has
no CUDA device, calls fail with an exception that says so.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "librosy_gb300.so")

RESULT_NAMES = {
    0: "ok", 1: "state_changed", 2: "error", 3: "invalid_argument", 4: "allocation_failure",
    5: "graphics_init_failure", 6: "graphics_frame_failure", 7: "graphics_swapchain_failure",
    8: "open_failed", 9: "write_failed", 10: "copy_failed", 11: "read_failed", 12: "create_failed",
    13: "update_failed", 14: "overflow", 15: "invalid_state", 16: "timeout",
}

# every symbol include/rosy_gb300.h declares
EXPORTS = [
    "rz_create", "rz_destroy", "rz_resize", "rz_set_asset", "rz_set_objects", "rz_update_objects",
    "rz_set_draw_config", "rz_update", "rz_render", "rz_sync", "rz_get_frame", "rz_read_frame",
    "rz_get_stats", "rz_get_stream", "rz_last_error", "rz_abi_version", "rz_set_stage_timing",
    "rz_get_stage_times", "rz_shadow_depth_static", "rz_add_scene", "rz_set_views", "rz_update_view",
    "rz_get_view_frame", "rz_set_tuning", "rz_get_tuning", "rz_autotune", "rz_set_gbuffer", "rz_get_view_gbuffer",
    "rz_set_debug_objects", "rz_set_wait_limit", "rz_upsampler_set_wait_limit", "rz_read_sync",
    "rz_upsampler_create", "rz_upsampler_destroy", "rz_upsampler_set_params", "rz_upsampler_get_params",
    "rz_upsampler_infer", "rz_upsampler_accumulate", "rz_upsampler_get_grads", "rz_upsampler_adam_step",
    "rz_upsampler_status", "rz_upsampler_selftest_gemm", "rz_rsy_read", "rz_rsy_free", "rz_rsy_get_info",
    "rz_rsy_get_meshes", "rz_rsy_get_materials", "rz_rsy_get_samplers", "rz_rsy_get_image", "rz_rsy_get_scene",
    "rz_dds_read", "rz_dds_parse", "rz_dds_free", "rz_dds_get_info", "rz_bc7_decode", "rz_bc7_decode_texture_unit",
]

_lib = None


class RzError(RuntimeError):
    def __init__(self, code: int, what: str, detail: str = ""):
        self.code = code
        super().__init__(f"{what}: {RESULT_NAMES.get(code, code)}" + (f" ({detail})" if detail else ""))


def load(build_if_missing: bool = False):
    """Returns the ctypes handle of librosy_gb300.so."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build
            build.build()
        else:
            raise RuntimeError(f"renderer library not built: {LIB_PATH} is missing (run rosy_gb300.build.build())")
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    u32 = C.c_uint32
    lib.rz_create.argtypes = [C.POINTER(P), C.POINTER(_abi.RzConfig)]
    lib.rz_destroy.argtypes = [P]
    lib.rz_destroy.restype = None
    lib.rz_resize.argtypes = [P, u32, u32]
    lib.rz_set_asset.argtypes = [P, P, u32, P, u32, P, u32, P, u32]
    lib.rz_set_objects.argtypes = [P, P, u32, P, u32]
    lib.rz_update_objects.argtypes = [P, u32, P, u32]
    lib.rz_set_draw_config.argtypes = [P, P]
    lib.rz_update.argtypes = [P, P]
    lib.rz_render.argtypes = [P]
    lib.rz_sync.argtypes = [P, u32]
    lib.rz_get_frame.argtypes = [P, C.POINTER(_abi.RzFrameOut)]
    lib.rz_read_frame.argtypes = [P, P, C.c_size_t, P, C.c_size_t]
    lib.rz_read_sync.argtypes = [P, u32, u32]
    lib.rz_read_sync.restype = C.c_int
    lib.rz_get_stats.argtypes = [P, C.POINTER(_abi.RzStats)]
    lib.rz_get_stream.argtypes = [P]
    lib.rz_get_stream.restype = P
    lib.rz_last_error.argtypes = [P]
    lib.rz_last_error.restype = C.c_char_p
    lib.rz_set_stage_timing.argtypes = [P, u32]
    lib.rz_get_stage_times.argtypes = [P, C.POINTER(C.c_float), u32, C.POINTER(u32)]
    lib.rz_shadow_depth_static.argtypes = [P, u32, P, u32, C.POINTER(C.c_float), C.POINTER(C.c_float), P, u32, u32,
                                           P, P]
    lib.rz_shadow_depth_static.restype = C.c_int
    lib.rz_add_scene.argtypes = [P, P, u32, P, u32, P, u32, P, u32, P, u32, P, u32, C.POINTER(u32)]
    lib.rz_set_views.argtypes = [P, P, u32]
    lib.rz_update_view.argtypes = [P, u32, P]
    lib.rz_get_view_frame.argtypes = [P, u32, C.POINTER(_abi.RzFrameOut)]
    lib.rz_set_tuning.argtypes = [P, C.POINTER(_abi.RzTuning)]
    lib.rz_get_tuning.argtypes = [P, C.POINTER(_abi.RzTuning)]
    lib.rz_autotune.argtypes = [P, u32, C.POINTER(_abi.RzTuning), C.POINTER(C.c_float), u32]
    lib.rz_set_wait_limit.argtypes = [P, u32]
    lib.rz_upsampler_set_wait_limit.argtypes = [P, C.c_uint64]
    for name in ("rz_add_scene", "rz_set_views", "rz_update_view", "rz_get_view_frame", "rz_set_tuning",
                 "rz_get_tuning", "rz_autotune", "rz_set_wait_limit", "rz_upsampler_set_wait_limit"):
        getattr(lib, name).restype = C.c_int
    G = C.POINTER(_abi.RzGbuffer)
    lib.rz_set_gbuffer.argtypes = [P, u32]
    lib.rz_set_debug_objects.argtypes = [P, P, u32]
    lib.rz_get_view_gbuffer.argtypes = [P, u32, G]
    lib.rz_upsampler_create.argtypes = [C.POINTER(P), C.c_int, u32, u32]
    lib.rz_upsampler_destroy.argtypes = [P]
    lib.rz_upsampler_destroy.restype = None
    lib.rz_upsampler_set_params.argtypes = [P, C.POINTER(C.c_float), u32, P]
    lib.rz_upsampler_get_params.argtypes = [P, C.POINTER(C.c_float), u32, P]
    lib.rz_upsampler_infer.argtypes = [P, G, P, P]
    lib.rz_upsampler_accumulate.argtypes = [P, G, P, P, P]
    lib.rz_upsampler_get_grads.argtypes = [P, C.POINTER(C.c_float), u32, C.POINTER(C.c_double),
                                           C.POINTER(C.c_uint64), P]
    lib.rz_upsampler_adam_step.argtypes = [P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, P]
    lib.rz_upsampler_status.argtypes = [P, C.POINTER(u32), P]
    lib.rz_upsampler_selftest_gemm.argtypes = [P, P, P, u32, u32, P]
    for name in ("rz_set_gbuffer", "rz_set_debug_objects", "rz_get_view_gbuffer", "rz_upsampler_create", "rz_upsampler_set_params",
                 "rz_upsampler_get_params", "rz_upsampler_infer", "rz_upsampler_accumulate", "rz_upsampler_get_grads",
                 "rz_upsampler_adam_step", "rz_upsampler_status", "rz_upsampler_selftest_gemm"):
        getattr(lib, name).restype = C.c_int
    lib.rz_rsy_read.argtypes = [C.c_char_p, C.POINTER(P)]
    lib.rz_rsy_free.argtypes = [P]
    lib.rz_rsy_free.restype = None
    lib.rz_rsy_get_info.argtypes = [P, C.POINTER(_abi.RzRsyInfo)]
    lib.rz_rsy_get_meshes.argtypes = [P, P, u32]
    lib.rz_rsy_get_materials.argtypes = [P, P, u32]
    lib.rz_rsy_get_samplers.argtypes = [P, P, u32]
    lib.rz_rsy_get_image.argtypes = [P, u32, C.POINTER(u32), C.c_char_p, u32, C.POINTER(u32)]
    lib.rz_rsy_get_scene.argtypes = [P, P, u32, P, u32]
    for name in ("rz_rsy_read", "rz_rsy_get_info", "rz_rsy_get_meshes", "rz_rsy_get_materials", "rz_rsy_get_samplers",
                 "rz_rsy_get_image", "rz_rsy_get_scene"):
        getattr(lib, name).restype = C.c_int
    lib.rz_dds_read.argtypes = [C.c_char_p, C.POINTER(P)]
    lib.rz_dds_parse.argtypes = [P, C.c_uint64, C.POINTER(P)]
    lib.rz_dds_free.argtypes = [P]
    lib.rz_dds_free.restype = None
    lib.rz_dds_get_info.argtypes = [P, C.POINTER(_abi.RzDdsInfo)]
    lib.rz_bc7_decode.argtypes = [P, u32, u32, P, P]
    lib.rz_bc7_decode_texture_unit.argtypes = [P, u32, u32, P]
    for name in ("rz_dds_read", "rz_dds_parse", "rz_dds_get_info", "rz_bc7_decode", "rz_bc7_decode_texture_unit"):
        getattr(lib, name).restype = C.c_int
    lib.rz_abi_version.argtypes = []
    lib.rz_abi_version.restype = u32
    for name in ("rz_create", "rz_resize", "rz_set_asset", "rz_set_objects", "rz_update_objects",
                 "rz_set_draw_config", "rz_update", "rz_render", "rz_sync", "rz_get_frame", "rz_read_frame",
                 "rz_get_stats", "rz_set_stage_timing", "rz_get_stage_times"):
        getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib
