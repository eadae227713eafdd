"""Batched views: several scenes and views of uneven size rendered by one
rz_render (one launch per stage over all views); every view must match the
oracle rendering that view alone, bit-exactly for visibility/depth/shadow."""
import numpy as np
import pytest

from rosy_gb300 import scene as sc
from rosy_gb300.graphics import Graphics
from test_gpu_parity import check_parity


def render_batch(scenes, views, samples=1, debug_objects=None):
    g = Graphics()
    g.init(64, 64, 64, samples=samples)
    try:
        idx = [g.add_scene(s) for s in scenes]
        g.set_views([(idx[k], v.width, v.height, v.shadow_size, v.draw_config) for k, v in views])
        if debug_objects is not None:
            g.set_debug_objects(debug_objects)
        for i, (_, v) in enumerate(views):
            g.update_view(i, v.scene)
        g.render()
        if g.sync_code() == 14:
            g.render()
        g.sync()
        return [g.download_view(i) for i in range(len(views))]
    finally:
        g.deinit()


@pytest.mark.gpu
def test_batched_views_match_single_view_oracle(gpu, oracle):
    scenes, views = sc.batch_views(seed=3, views=7, scenes=3, min_tris=500, max_tris=6000, min_size=40,
                                   max_size=260, min_shadow=128, max_shadow=512, texture_size=32)
    outs = render_batch(scenes, views)
    for (k, v), out in zip(views, outs):
        check_parity(v, oracle.render(v), out)


@pytest.mark.gpu
def test_batch_with_blended_and_mixed_state(gpu, oracle):
    a = sc.with_blended(sc.random_triangles(seed=21, triangles=300, width=64, height=64, shadow_size=128,
                                            texture_size=32), 0.4)
    b = sc.random_triangles(seed=22, triangles=500, width=64, height=64, shadow_size=128, texture_size=32,
                            pcf_mode=sc.PCF_3X3)
    v1 = sc.view_of(a, 96, 70, 160)
    v2 = sc.view_of(b, 50, 120, 256)
    v2.draw_config = v2.draw_config.copy()
    v2.draw_config["cull_enabled"] = 0
    v3 = sc.view_of(a, 130, 40, 96)
    outs = render_batch([a, b], [(0, v1), (1, v2), (0, v3)])
    for v, out in zip((v1, v2, v3), outs):
        check_parity(v, oracle.render(v), out)


@pytest.mark.gpu
def test_sequential_launches_equal_batched_and_autotune(gpu, oracle):
    scenes, views = sc.batch_views(seed=5, views=6, scenes=2, min_tris=400, max_tris=4000, min_size=40,
                                   max_size=200, min_shadow=128, max_shadow=384, texture_size=32)
    g = Graphics()
    g.init(64, 64, 64)
    try:
        idx = [g.add_scene(s) for s in scenes]
        g.set_views([(idx[k], v.width, v.height, v.shadow_size, v.draw_config) for k, v in views])
        for i, (_, v) in enumerate(views):
            g.update_view(i, v.scene)
        g.render()
        if g.sync_code() == 14:
            g.render()
        g.sync()
        batched = [g.download_view(i) for i in range(len(views))]
        g.set_tuning(batched=False)
        g.render()
        g.sync()
        seq = [g.download_view(i) for i in range(len(views))]
        for a, b in zip(batched, seq):
            for k in ("ids", "color"):
                assert np.array_equal(a[k], b[k])
            for k in ("depth", "shadow"):
                assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32))
        g.set_tuning(batched=True)
        chosen, ms = g.autotune(frames=2)
        assert chosen["chunk_stamps"] in (16, 32, 64) and chosen["small_extent"] in (4, 8, 12)
        assert all(m > 0 for m in ms)
        g.render()
        g.sync()
        for (k, v), i in zip(views, range(len(views))):
            check_parity(v, oracle.render(v), g.download_view(i))
    finally:
        g.deinit()


@pytest.mark.gpu
def test_batch_with_msaa_cascades_and_blending(gpu, oracle):
    """Features together: a 4x multisampled context whose views have different
    numbers of shadow cascades (1, 2, 4), one with blended surfaces; every view
    against the oracle rendering it alone (per-sample ids and depths bit-exact)."""
    a = sc.with_blended(sc.random_triangles(seed=41, triangles=300, width=64, height=64, shadow_size=128,
                                            texture_size=32), 0.4)
    b = sc.random_triangles(seed=42, triangles=500, width=64, height=64, shadow_size=128, texture_size=32)
    views = []
    for k, (src, w, h, sz, n) in enumerate([(a, 90, 64, 128, 1), (b, 72, 100, 160, 2), (a, 120, 48, 96, 4)]):
        v = sc.view_of(src, w, h, sz, camera=k)
        P = v.scene["shadow_projection_near"][0].reshape(4, 4).copy()
        P[:, 0:2] *= 16.0  # small light extent: the geometry spans several cascades
        v.scene = v.scene.copy()
        v.scene["shadow_projection_near"] = P.reshape(1, 16)
        v.cameras = [v.scene]
        v.draw_config = v.draw_config.copy()
        v.draw_config["shadow_cascades"] = n
        v.samples = 4
        views.append((0 if src is a else 1, v))
    outs = render_batch([a, b], views, samples=4)
    for (_, v), out in zip(views, outs):
        ref = oracle.render(v)
        assert np.array_equal(out["ids"], ref["ids"])
        assert np.array_equal(out["vis_depth"].view(np.uint32), ref["depth"].view(np.uint32))
        assert np.array_equal(out["shadow"].view(np.uint32), ref["shadow"].view(np.uint32))
        d = np.abs(out["color"].astype(np.int32) - ref["color"].astype(np.int32))
        assert d.max() <= 1, d.max()
