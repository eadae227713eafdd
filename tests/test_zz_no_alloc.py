"""The shadow depth entry point that allocates nothing (rz_shadow_depth_static).

Callers that cannot allocate device memory while running (engines with their
own allocator or a fixed memory budget, frame loops that must not call
cudaMalloc/cudaFree) use this entry point; its scratch is a fixed array
compiled into the library. This file is collected last so that a failure here
comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from rosy_gb300 import _lib
from rosy_gb300 import scene as sc
from rosy_gb300.graphics import render_scene

RZ_OK, RZ_INVALID_ARGUMENT = 0, 3


def _static_shadow(lib, s, torch, depth):
    pos = np.zeros((len(s.vertices), 4), np.float32)
    pos[:, :3] = s.vertices[:, 0:3]
    d_pos = torch.from_numpy(pos).cuda()
    d_idx = torch.from_numpy(s.indices.astype(np.int64)).to(torch.int32).cuda()
    proj = (C.c_float * 16)(*s.scene["shadow_projection_near"][0].tolist())
    world = (C.c_float * 16)(*s.objects[0, 0:16].tolist())
    dc = np.ascontiguousarray(s.draw_config)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.rz_shadow_depth_static(d_pos.data_ptr(), len(pos), d_idx.data_ptr(), len(s.indices), proj, world,
                                    dc.ctypes.data, s.shadow_size, s.shadow_size, depth.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc


@pytest.mark.gpu
def test_static_shadow_pass_matches_render_twice(gpu):
    """Two calls in a row through the C ABI match rz_render's shadow map bit for bit."""
    import torch

    s = sc.random_triangles(seed=11, triangles=600, width=160, height=96, shadow_size=256, texture_size=32)
    # a light that sees the whole mesh large in the map
    s.scene["shadow_projection_near"] = sc.colmajor(
        np.diag([0.9, 0.9, -0.2, 1.0]) @ np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, -3.0], [0, 0, 0, 1.0]]))
    ref = render_scene(s)["shadow"]
    assert (ref > 0).mean() > 0.05
    lib = _lib.load()
    for _ in range(2):
        depth = torch.full((s.shadow_size, s.shadow_size), 0.5, dtype=torch.float32, device="cuda")
        assert _static_shadow(lib, s, torch, depth) == RZ_OK
        got = depth.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.gpu
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
