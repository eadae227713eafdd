"""CPU checks of the C ABI: the library builds, loads, and exports every symbol
include/rosy_gb300.h declares; the ctypes mirror has the header's layouts."""
import ctypes as C
import os
import re

import numpy as np

from rosy_gb300 import _abi, _lib
from rosy_gb300 import scene as sc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "rosy_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rz_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_bound_symbols():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(renderer_lib):
    for name in declared_functions():
        assert hasattr(renderer_lib, name), name
    assert renderer_lib.rz_abi_version() == 2


def test_record_layouts():
    assert C.sizeof(_abi.RzVertex) == 64
    assert sc.OBJECT_FLOATS * 4 == 164
    assert sc.SCENE_DTYPE.itemsize == 408
    assert sc.SURFACE_DTYPE.itemsize == 28
    assert sc.SAMPLER_DTYPE.itemsize == 8
    assert sc.DRAW_CONFIG_DTYPE.itemsize == 32
    assert C.sizeof(_abi.RzConfig) == 32
    assert C.sizeof(_abi.RzFrameOut) == 48
    assert C.sizeof(_abi.RzStats) == 40


def test_header_compiles_as_c_and_matches_sizes(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text(
        '#include "rosy_gb300.h"\n#include <stdio.h>\n'
        'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(rz_vertex), sizeof(rz_object),'
        ' sizeof(rz_scene_data), sizeof(rz_surface), sizeof(rz_material), sizeof(rz_sampler),'
        ' sizeof(rz_draw_config), sizeof(rz_texture), sizeof(rz_mesh), sizeof(rz_dds_info));'
        ' printf("%zu\\n", sizeof(rz_debug_object)); return 0;}\n')
    exe = tmp_path / "sizes"
    import subprocess

    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert [int(x) for x in got] == [64, 164, 408, 28, sc.MATERIAL_DTYPE.itemsize, 8, 32, 32, 24, 40,
                                     sc.DEBUG_OBJECT_DTYPE.itemsize]


def test_calls_without_a_context_are_rejected(renderer_lib):
    P = C.c_void_p
    assert renderer_lib.rz_render(None) == 3
    assert renderer_lib.rz_sync(None, 0) == 3
    assert renderer_lib.rz_set_debug_objects(None, None, 0) == 3
    assert renderer_lib.rz_read_frame(None, None, 0, None, 0) == 3
    assert renderer_lib.rz_read_sync(None, 0, 0) == 3
    assert renderer_lib.rz_get_frame(None, None) == 3
    out = C.c_void_p()
    assert renderer_lib.rz_create(C.byref(out), None) == 3
    renderer_lib.rz_destroy(None)


def test_create_rejects_bad_config_without_touching_the_gpu(renderer_lib):
    out = C.c_void_p()
    cfg = _abi.RzConfig(width=0, height=10, shadow_map_size=16, samples=1, device=0)
    assert renderer_lib.rz_create(C.byref(out), C.byref(cfg)) == 3
    cfg = _abi.RzConfig(width=10, height=10, shadow_map_size=16, samples=3, device=0)
    assert renderer_lib.rz_create(C.byref(out), C.byref(cfg)) == 3


def test_texture_entry_points_reject_bad_arguments_without_touching_the_gpu(renderer_lib):
    """BC7 decode and .dds entry points validate their arguments before any CUDA call."""
    buf = C.create_string_buffer(64)
    assert renderer_lib.rz_bc7_decode(None, 4, 4, buf, None) == 3
    assert renderer_lib.rz_bc7_decode(buf, 4, 4, None, None) == 3
    assert renderer_lib.rz_bc7_decode(buf, 0, 4, buf, None) == 3
    assert renderer_lib.rz_bc7_decode_texture_unit(buf, 6, 4, buf) == 3  # not a multiple of 4
    assert renderer_lib.rz_bc7_decode_texture_unit(None, 4, 4, buf) == 3
    out = C.c_void_p()
    assert renderer_lib.rz_dds_read(None, C.byref(out)) == 3
    assert renderer_lib.rz_dds_parse(None, 16, C.byref(out)) == 3
    assert renderer_lib.rz_dds_get_info(None, None) == 3
    renderer_lib.rz_dds_free(None)


def test_marshalling_rejects_ranges_outside_their_arrays():
    """The library reads meshes and texels through raw pointers, so the Python side
    checks every range against its array before handing the pointers over."""
    import dataclasses

    import pytest

    s = sc.tiny(0)
    _abi.Marshalled(s)  # the scene as made is accepted
    bad = dataclasses.replace(s, meshes=[(0, len(s.vertices) + 1, 0, len(s.indices))])
    with pytest.raises(ValueError, match="mesh 0"):
        _abi.Marshalled(bad)
    bad = dataclasses.replace(s, meshes=[(0, len(s.vertices), 3, len(s.indices))])
    with pytest.raises(ValueError, match="mesh 0"):
        _abi.Marshalled(bad)
    t = s.textures[0]
    short = dataclasses.replace(t, texels=t.texels[:-1])
    with pytest.raises(ValueError, match="texture 0"):
        _abi.Marshalled(dataclasses.replace(s, textures=[short] + s.textures[1:]))
    huge = dataclasses.replace(t, width=1 << 31, height=1, levels=1)
    with pytest.raises(ValueError, match="texture 0"):
        _abi.Marshalled(dataclasses.replace(s, textures=[huge] + s.textures[1:]))
    # BC7 chains are counted in 16-byte blocks
    assert _abi.texel_bytes(6, 5, 3, _abi.TEXELS_BC7) == (2 * 2 + 1 * 1 + 1 * 1) * 16
    assert _abi.texel_bytes(6, 5, 3, _abi.TEXELS_RGBA8) == (30 + 6 + 1) * 4
