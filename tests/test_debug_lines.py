"""Known-answer tests of the debug-line overlay in the oracle (DRAW DEBUG,
src/Engine/Graphics.cpp:5694-5738; vertex stage src/shaders/debug.slang:5-35).

Lines are 5 pixels wide rectangles (Vulkan strict lines) sampled at pixel
centres, or at the four standard sample positions with 4x multisampling; a
sample on a long edge belongs to the line on the +perp side only, the end
point is excluded. Depth is tested GREATER_OR_EQUAL against the opaque depth
and never written; later segments cover earlier ones.
"""
import math

import numpy as np
import pytest

from kat_scenes import flat_scene, ndc
from rosy_gb300 import scene as sc

RED, GREEN = (1.0, 0.0, 0.0, 1.0), (0.0, 1.0, 0.0, 1.0)


def seg_transform(a, b):
    """World transform taking the table's line (0,0,0)-(0,0,1) to a -> b."""
    return np.array([[1, 0, b[0] - a[0], a[0]], [0, 1, b[1] - a[1], a[1]],
                     [0, 0, b[2] - a[2], a[2]], [0, 0, 0, 1]], np.float64)


def window_line(a, b, W, H, z=(0.5, 0.5)):
    """Transform of a line between window positions a and b (with identity view-projection)."""
    (ax, ay), (bx, by) = ndc(a[0], a[1], W, H), ndc(b[0], b[1], W, H)
    return seg_transform((ax, ay, z[0]), (bx, by, z[1]))


def with_lines(s, objs, samples=1):
    s.debug_objects = np.concatenate(objs)
    s.samples = samples
    return s


def painted(out, rgb):
    return np.all(out["color"][..., :3] == np.array(rgb, np.uint8), axis=-1)


def background_scene(W=32, H=16):
    # one small triangle in a corner, so the frame is mostly background
    return flat_scene([((0.5, 0.5, 0.5), (2.5, 0.5, 0.5), (0.5, 2.5, 0.5))], W=W, H=H)


def test_screen_space_line_is_five_pixels_wide(oracle):
    W, H = 32, 16
    s = background_scene(W, H)
    # flags 1: z = w = 1, so the line is in front of everything
    with_lines(s, [sc.debug_object(sc.DEBUG_LINE, window_line((8, 8), (24, 8), W, H), RED, sc.DEBUG_SCREEN_SPACE)])
    m = painted(oracle.render(s, threads=1), (255, 0, 0))
    expected = np.zeros((H, W), bool)
    expected[6:11, 8:24] = True  # centres 5.5 (perp = -2.5 px) out, 10.5 (+2.5 px) in; end x = 24 excluded
    assert np.array_equal(m, expected)


def test_world_space_line_depth_test_against_the_opaque_surface(oracle):
    W, H = 32, 16
    # a wall at depth 0.5 over the right half
    s = flat_scene([((16, 0, 0.5), (32, 0, 0.5), (32, 16, 0.5)), ((16, 0, 0.5), (32, 16, 0.5), (16, 16, 0.5))],
                   W=W, H=H)
    behind = window_line((4, 4), (28, 4), W, H, z=(0.25, 0.25))   # reverse-Z: smaller is farther
    front = window_line((4, 12), (28, 12), W, H, z=(0.75, 0.75))
    equal = window_line((4, 8), (28, 8), W, H, z=(0.5, 0.5))      # GREATER_OR_EQUAL passes
    with_lines(s, [sc.debug_object(sc.DEBUG_LINE, t, RED) for t in (behind, front, equal)])
    out = oracle.render(s, threads=1)
    m = painted(out, (255, 0, 0))
    assert m[4, 4:16].all() and not m[4, 16:28].any()
    assert m[12, 4:28].all() and m[8, 4:28].all()
    # the overlay writes no depth and no triangle ids
    ref = oracle.render(flat_scene([((16, 0, 0.5), (32, 0, 0.5), (32, 16, 0.5)),
                                    ((16, 0, 0.5), (32, 16, 0.5), (16, 16, 0.5))], W=W, H=H), threads=1)
    assert np.array_equal(out["depth"], ref["depth"]) and np.array_equal(out["ids"], ref["ids"])


def test_later_segments_cover_earlier_ones(oracle):
    W, H = 32, 32
    s = background_scene(W, H)
    h = sc.debug_object(sc.DEBUG_LINE, window_line((4, 16), (28, 16), W, H), RED, sc.DEBUG_SCREEN_SPACE)
    v = sc.debug_object(sc.DEBUG_LINE, window_line((16, 4), (16, 28), W, H), GREEN, sc.DEBUG_SCREEN_SPACE)
    a = oracle.render(with_lines(background_scene(W, H), [h, v]), threads=1)
    b = oracle.render(with_lines(s, [v, h]), threads=1)
    assert painted(a, (0, 255, 0))[16, 16] and painted(b, (255, 0, 0))[16, 16]
    assert painted(a, (255, 0, 0))[16, 6] and painted(b, (0, 255, 0))[6, 16]


def test_multisampled_line_covers_samples(oracle):
    W, H = 32, 16
    s = with_lines(background_scene(W, H),
                   [sc.debug_object(sc.DEBUG_LINE, window_line((8, 8), (24, 8), W, H), RED, sc.DEBUG_SCREEN_SPACE)],
                   samples=4)
    out = oracle.render(s, threads=1)
    full = painted(out, (255, 0, 0))
    assert full[6:10, 8:24].all() and not full[5].any() and not full[10].any()
    # rows 5 and 10: two of the four samples (y offsets 160/224 and 32/96 of 256) are on the line
    bg = oracle.render(background_scene(W, H), threads=1)["color"][5, 12]
    for row in (5, 10):
        px = out["color"][row, 12]
        assert px[0] > bg[0] and 0 < px[0] < 255, (row, px)
        assert np.array_equal(out["color"][row, 8:24], np.repeat(px[None], 16, 0))


def test_line_is_clipped_at_the_near_plane(oracle):
    W, H = 32, 16
    # clip z from 0.5 to 1.5 with w = 1: the near plane z <= w keeps the first half
    (ax, ay), (bx, by) = ndc(8, 8, W, H), ndc(24, 8, W, H)
    t = seg_transform((ax, ay, 0.5), (bx, by, 1.5))
    out = oracle.render(with_lines(background_scene(W, H), [sc.debug_object(sc.DEBUG_LINE, t, RED)]), threads=1)
    m = painted(out, (255, 0, 0))
    expected = np.zeros((H, W), bool)
    expected[6:11, 8:16] = True
    assert np.array_equal(m, expected)


def test_line_outside_the_view_draws_nothing(oracle):
    W, H = 32, 16
    behind_far = seg_transform((-0.5, 0, -0.5), (0.5, 0, -0.25))  # z < 0: beyond the far plane
    out = oracle.render(with_lines(background_scene(W, H), [sc.debug_object(sc.DEBUG_LINE, behind_far, RED)]),
                        threads=1)
    assert not painted(out, (255, 0, 0)).any()


def test_transform_is_points_and_cross(oracle):
    W, H = 32, 16
    (ax, ay), (bx, by) = ndc(8, 8, W, H), ndc(24, 8, W, H)
    pts = np.zeros((4, 4))
    pts[:, 0] = (ax, ay, 0.5, 1.0)  # columns 0 and 1 are the segment's ends
    pts[:, 1] = (bx, by, 0.5, 1.0)
    p = sc.debug_object(sc.DEBUG_LINE, pts, RED, sc.DEBUG_TRANSFORM_IS_POINTS)
    q = sc.debug_object(sc.DEBUG_CROSS, window_line((8, 8), (24, 8), W, H), RED)  # a cross draws the line
    a = painted(oracle.render(with_lines(background_scene(W, H), [p]), threads=1), (255, 0, 0))
    b = painted(oracle.render(with_lines(background_scene(W, H), [q]), threads=1), (255, 0, 0))
    expected = np.zeros((H, W), bool)
    expected[6:11, 8:24] = True
    assert np.array_equal(a, expected) and np.array_equal(b, expected)


def test_screen_space_circle(oracle):
    W, H = 64, 32
    # screen space: transform * (x, y * W/H, z, w). x: 0.25 NDC = 8 px; y: 0.25 * W/H = 0.5 NDC = 8 px
    t = np.diag([0.25, 0.25, 1.0, 1.0])
    out = oracle.render(with_lines(background_scene(W, H), [sc.debug_object(sc.DEBUG_CIRCLE, t, RED,
                                                                            sc.DEBUG_SCREEN_SPACE)]), threads=1)
    m = painted(out, (255, 0, 0))
    # a ring of radius 8 px around the centre (32, 16), 5 px wide; the centre untouched
    assert not m[16, 32] and m.sum() > 150
    ys, xs = np.nonzero(m)
    r = np.hypot(xs + 0.5 - 32, ys + 0.5 - 16)
    assert r.min() >= 8 - 2.5 - 0.3 and r.max() <= 8 + 2.5 + 0.3
    # 50 chords of the unit circle: every direction is drawn
    ang = np.arctan2(ys + 0.5 - 16, xs + 0.5 - 32)
    assert np.histogram(ang, bins=16, range=(-math.pi, math.pi))[0].min() > 0


def test_fp64_output_carries_the_overlay(oracle):
    W, H = 32, 16
    s = with_lines(background_scene(W, H),
                   [sc.debug_object(sc.DEBUG_LINE, window_line((8, 8), (24, 8), W, H), (0.25, 0.5, 0.75, 1.0),
                                    sc.DEBUG_SCREEN_SPACE)])
    out = oracle.render(s, threads=1, fp64=True)
    srgb = [c * 12.92 if c <= 0.0031308 else 1.055 * c ** (1 / 2.4) - 0.055 for c in (0.25, 0.5, 0.75)]
    assert np.allclose(out["color_f64"][8, 12, :3], srgb) and out["color_f64"][8, 12, 3] == 1.0


@pytest.mark.parametrize("vertical", [False, True])
def test_axis_aligned_lines_are_five_pixels_wide_at_any_offset(oracle, vertical):
    """The half-open band (c - 2.5, c + 2.5] holds exactly five pixel centres wherever the
    line lies, and the ends cover the centres in [x0, x1)."""
    W, H = 48, 48
    rng = np.random.default_rng(7)
    objs, spans = [], []
    for i in range(6):
        c = 6.0 + 7.0 * i + rng.integers(0, 256) / 256.0  # exact in 1/256 pixel
        x0 = 4.0 + rng.integers(0, 256) / 256.0
        x1 = x0 + 20.0 + rng.integers(0, 2048) / 256.0
        a, b = ((c, x0), (c, x1)) if vertical else ((x0, c), (x1, c))
        objs.append(sc.debug_object(sc.DEBUG_LINE, window_line(a, b, W, H), (1.0, 0.0, 0.0, 1.0),
                                    sc.DEBUG_SCREEN_SPACE))
        spans.append((c, x0, x1))
    for (c, x0, x1), o in zip(spans, objs):
        out = oracle.render(with_lines(background_scene(W, H), [o]), threads=1)
        m = painted(out, (255, 0, 0))
        if vertical:
            m = m.T
        rows = np.nonzero(m.any(axis=1))[0]
        cols = np.nonzero(m.any(axis=0))[0]
        # perp > 0 on the side of larger y for a line running towards +x; towards +y it is the side of
        # smaller x, so the included edge swaps between the two cases
        if vertical:
            assert rows.tolist() == [r for r in range(W) if -2.5 <= (r + 0.5) - c < 2.5]
        else:
            assert rows.tolist() == [r for r in range(H) if -2.5 < (r + 0.5) - c <= 2.5]
        assert cols.tolist() == [k for k in range(W) if x0 <= k + 0.5 < x1]
        assert m[rows][:, cols].all()


def test_reversed_segment_covers_the_same_interior(oracle):
    """Swapping a segment's ends changes only the tie rules at its ends and edges."""
    W, H = 40, 40
    rng = np.random.default_rng(3)
    for _ in range(5):
        a = rng.uniform(5, 35, 2)
        b = rng.uniform(5, 35, 2)
        f = sc.debug_object(sc.DEBUG_LINE, window_line(a, b, W, H), RED, sc.DEBUG_SCREEN_SPACE)
        r = sc.debug_object(sc.DEBUG_LINE, window_line(b, a, W, H), RED, sc.DEBUG_SCREEN_SPACE)
        mf = painted(oracle.render(with_lines(background_scene(W, H), [f]), threads=1), (255, 0, 0))
        mr = painted(oracle.render(with_lines(background_scene(W, H), [r]), threads=1), (255, 0, 0))
        ys, xs = np.nonzero(mf ^ mr)
        if len(xs):  # only centres on the rectangle's boundary can differ
            p = np.stack([xs + 0.5, ys + 0.5], 1)
            d = b - a
            along = (p - a) @ d / (d @ d)
            perp = np.abs((p - a) @ np.array([-d[1], d[0]])) / np.linalg.norm(d)
            on_edge = (np.abs(perp - 2.5) < 0.01) | (np.abs(along) < 0.01) | (np.abs(along - 1) < 0.01)
            assert on_edge.all()


def test_view_space_uses_proj_without_a_divide(oracle):
    """flags 2: (proj * transform) * v, then z = w = 1; with an identity proj a line lands where the
    screen-space line does, and a scaled proj scales it without dividing by the original w."""
    W, H = 32, 16
    t = window_line((8, 8), (24, 8), W, H)
    s = background_scene(W, H)
    s.scene = s.scene.copy()
    s.scene["proj"] = sc.colmajor(np.eye(4))
    a = painted(oracle.render(with_lines(s, [sc.debug_object(sc.DEBUG_LINE, t, RED, sc.DEBUG_VIEW_SPACE)]),
                              threads=1), (255, 0, 0))
    expected = np.zeros((H, W), bool)
    expected[6:11, 8:24] = True
    assert np.array_equal(a, expected)
    # w = 2 in the proj's last row would halve x and y after a divide; the shader sets w = 1 instead
    p = np.eye(4)
    p[3, 3] = 2.0
    s.scene["proj"] = sc.colmajor(p)
    b = painted(oracle.render(with_lines(s, [sc.debug_object(sc.DEBUG_LINE, t, RED, sc.DEBUG_VIEW_SPACE)]),
                              threads=1), (255, 0, 0))
    assert np.array_equal(b, expected)
