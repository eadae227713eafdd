"""Failure paths on the GPU, injected from the host (no device fault is ever caused)."""
import numpy as np
import pytest

from rosy_gb300 import scene as sc
from rosy_gb300._lib import RzError
from rosy_gb300.graphics import Graphics
from test_gpu_parity import check_parity

RZ_INVALID_ARGUMENT, RZ_OVERFLOW, RZ_INVALID_STATE = 3, 14, 15


@pytest.mark.gpu
def test_work_queue_overflow_is_reported_then_grows(gpu, oracle):
    s = sc.random_triangles(seed=2, triangles=600, width=256, height=160, shadow_size=256, texture_size=64)
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size, queue_chunks=4)  # far too small a queue
    try:
        g.set_asset(s)
        g.set_graphic_objects(s.objects, s.surfaces)
        g.set_draw_config(s.draw_config)
        g.update(s.scene)
        g.render()
        assert g.sync_code() == RZ_OVERFLOW
        assert g.stats().error_flags != 0
        g.render()  # the queue has grown
        g.sync()
        assert g.stats().error_flags == 0
        check_parity(s, oracle.render(s), g.download())
    finally:
        g.deinit()


@pytest.mark.gpu
def test_invalid_inputs_are_rejected(gpu):
    s = sc.tiny(0)
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size)
    try:
        with pytest.raises(RzError) as e:
            g.render()
        assert e.value.code == RZ_INVALID_STATE
        bad = sc.tiny(0)
        bad.indices = bad.indices.copy()
        bad.indices[5] = 10 ** 6  # index outside its mesh
        with pytest.raises(RzError) as e:
            g.set_asset(bad)
        assert e.value.code == RZ_INVALID_ARGUMENT
        g.set_asset(s)
        surf = s.surfaces.copy()
        surf["mesh_index"] = 7
        with pytest.raises(RzError) as e:
            g.set_graphic_objects(s.objects, surf)
        assert e.value.code == RZ_INVALID_ARGUMENT
        with pytest.raises(RzError) as e:
            g.set_graphic_objects(s.objects[:0], s.surfaces)
        assert e.value.code == RZ_INVALID_ARGUMENT
        surf = s.surfaces.copy()
        surf["index_count"] = len(s.indices) + 3
        with pytest.raises(RzError) as e:
            g.set_graphic_objects(s.objects, surf)
        assert e.value.code == RZ_INVALID_ARGUMENT
        g.set_graphic_objects(s.objects, s.surfaces)
        g.update(s.scene)
        g.render()
        g.sync(timeout_ms=10000)
    finally:
        g.deinit()


@pytest.mark.gpu
def test_stage_timing(gpu):
    s = sc.tiny(1)
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size)
    try:
        g.set_asset(s)
        g.set_graphic_objects(s.objects, s.surfaces)
        g.update(s.scene)
        g.set_stage_timing(True)
        g.render()
        g.sync()
        t = g.stage_times()
        assert set(t) == set(Graphics.STAGES) and all(v >= 0 for v in t.values())
        g.set_stage_timing(False)
        g.render()
        g.sync()
    finally:
        g.deinit()


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [1, 4])
def test_launch_count_is_exact(gpu, samples):
    """kernel_launches counts what the launchers enqueued: for one opaque view, the shadow
    prep (with the pass's clear) / setup / raster, the camera prep (with its clear) /
    setup, one raster per sample, the vertex stage and the shading; the same through the
    frame graph, a replay of it, and the stage-timed direct launches."""
    s = sc.tiny(2)
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size, samples=samples)
    try:
        g.set_asset(s)
        g.set_graphic_objects(s.objects, s.surfaces)
        g.update(s.scene)
        expected = 3 + 2 + samples + 1 + 1
        for timed in (False, False, True):
            g.set_stage_timing(timed)
            g.render()
            g.sync()
            assert g.stats().kernel_launches == expected
    finally:
        g.deinit()
