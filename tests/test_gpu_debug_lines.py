"""GPU parity of the debug-line overlay (DRAW DEBUG, src/Engine/Graphics.cpp:5694-5738)
against the oracle: the frame's ids, depth and shadow maps bit-exact (the overlay writes
none of them), colour within 1/255, and the pixels the overlay paints identical."""
import numpy as np
import pytest

from kat_scenes import flat_scene, ndc
from rosy_gb300 import scene as sc
from rosy_gb300.graphics import Graphics, render_scene
from test_gpu_batch import render_batch
from test_gpu_parity import check_parity


def seg(a, b):
    t = np.eye(4)
    t[:3, 2] = np.subtract(b, a)
    t[:3, 3] = a
    return t


def kat_scene(samples):
    W, H = 48, 32
    s = flat_scene([((24, 0, 0.5), (48, 0, 0.5), (48, 32, 0.5)), ((24, 0, 0.5), (48, 32, 0.5), (24, 32, 0.5))],
                   W=W, H=H)
    (ax, ay), (bx, by) = ndc(4, 6, W, H), ndc(44, 6, W, H)
    (cx, cy), (dx, dy) = ndc(4, 26, W, H), ndc(44, 20, W, H)
    pts = np.ones((4, 4))
    pts[:3, 0] = (*ndc(6, 2, W, H), 0.6)
    pts[:3, 1] = (*ndc(40, 30, W, H), 0.4)
    s.debug_objects = np.concatenate([
        sc.debug_object(sc.DEBUG_LINE, seg((ax, ay, 0.25), (bx, by, 0.25)), (1, 0, 0, 1)),    # behind the wall
        sc.debug_object(sc.DEBUG_LINE, seg((cx, cy, 0.75), (dx, dy, 0.75)), (0, 1, 0, 1)),    # in front
        sc.debug_object(sc.DEBUG_CROSS, seg((ax, ay, 0.5), (dx, dy, 1.5)), (0, 0, 1, 1)),     # near-clipped
        sc.debug_object(sc.DEBUG_CIRCLE, np.diag([0.3, 0.3, 1, 1]), (1, 1, 0, 1), sc.DEBUG_SCREEN_SPACE),
        sc.debug_object(sc.DEBUG_LINE, pts, (0, 1, 1, 1), sc.DEBUG_TRANSFORM_IS_POINTS),
    ])
    s.samples = samples
    return s


def without_overlay(s):
    t = sc.Scene(**{k: getattr(s, k) for k in s.__dataclass_fields__})
    t.debug_objects = None
    return t


def check_overlay(s, oracle, out):
    """check_parity, and with one sample per pixel the pixels the overlay paints (where the
    oracle's frame differs from its frame without the overlay) identical."""
    ref = oracle.render(s)
    if s.samples == 4:  # per-sample visibility; the depth output is sample 0's
        assert np.array_equal(out["ids"], ref["ids"])
        assert np.array_equal(out["vis_depth"].view(np.uint32), ref["depth"].view(np.uint32)), "sample depth differs"
        assert np.array_equal(out["depth"].view(np.uint32), ref["depth"][0].view(np.uint32)), "depth output differs"
        assert np.array_equal(out["shadow"].view(np.uint32), ref["shadow"].view(np.uint32))
        d = np.abs(out["color"].astype(np.int32) - ref["color"].astype(np.int32))
        assert d.max() <= 1, f"colour differs by {d.max()} at {np.count_nonzero(d > 1)} channels"
    else:
        check_parity(s, ref, out)
    painted = np.any(ref["color"] != oracle.render(without_overlay(s))["color"], axis=-1)
    assert painted.sum() > 0
    if s.samples == 1:  # fully covered pixels take the line's colour exactly
        assert np.array_equal(out["color"][painted], ref["color"][painted]), "overlay pixels differ"


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [1, 4])
def test_overlay_known_answer_scene(gpu, oracle, samples):
    s = kat_scene(samples)
    check_overlay(s, oracle, render_scene(s))


def _random(samples, blended):
    s = sc.random_triangles(seed=5 + samples, triangles=600, width=200, height=120, shadow_size=128, texture_size=32)
    if blended:
        s = sc.with_blended(s, 0.4)
    s.samples = samples
    s.debug_objects = sc.random_debug_objects(samples * 10 + blended, 48)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("samples,blended", [(1, False), (4, False), (1, True), (4, True)])
def test_overlay_random_objects(gpu, oracle, samples, blended):
    s = _random(samples, blended)
    check_overlay(s, oracle, render_scene(s))


@pytest.mark.gpu
def test_overlay_updates_in_place_and_turns_off(gpu, oracle):
    s = sc.random_triangles(seed=9, triangles=500, width=160, height=96, shadow_size=128, texture_size=32)
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size)
    try:
        g.set_asset(s)
        g.set_graphic_objects(s.objects, s.surfaces)
        g.set_draw_config(s.draw_config)
        g.update(s.scene)
        for seed, n in ((1, 24), (2, 24), (3, 31), (None, 0)):  # same count (in place), new count, off
            objs = None if seed is None else sc.random_debug_objects(seed, n)
            g.set_debug_objects(objs)
            g.render()
            g.sync()
            s.debug_objects = objs
            check_parity(s, oracle.render(s), g.download())
        assert g.stats().kernel_launches == 8  # overlay off: the plain single-sample frame again
    finally:
        g.deinit()


@pytest.mark.gpu
def test_overlay_in_batched_views(gpu, oracle):
    a = sc.random_triangles(seed=31, triangles=400, width=64, height=64, shadow_size=128, texture_size=32)
    b = sc.with_blended(sc.random_triangles(seed=32, triangles=300, width=64, height=64, shadow_size=128,
                                            texture_size=32), 0.3)
    views = [(0, sc.view_of(a, 120, 80, 128)), (1, sc.view_of(b, 72, 100, 160)), (0, sc.view_of(a, 90, 50, 96))]
    objs = sc.random_debug_objects(7, 40)
    outs = render_batch([a, b], views, debug_objects=objs)
    for (_, v), out in zip(views, outs):
        v.debug_objects = objs
        check_parity(v, oracle.render(v), out)
