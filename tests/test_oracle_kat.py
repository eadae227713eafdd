"""Known-answer tests that pin the CPU oracle (the reference ships no tests or
golden data, so these hand-derived cases are the pin).

Rules under test (Vulkan specification, as the reference's fixed-function state
sets them up in src/Engine/Graphics.cpp:4989-5040, 5195-5292, 5566-5691):
top-left fill rule with 8-bit sub-pixel snapping, front-face/culling, clipping,
GREATER_OR_EQUAL depth test in submission order, depth bias, sRGB/RGBA16F
output conversion, and mip-level selection.
"""
import math

import numpy as np
import pytest

from kat_scenes import flat_scene, one_surface_per_triangle
from rosy_gb300 import scene as sc


def coverage(o, s):
    return o.raster(s, threads=1)["ids"] > 0


def test_top_left_rule_shared_diagonal(oracle):
    # square with corners on pixel centres, split along its diagonal
    a, b, c, d = (1.5, 1.5, 0.5), (5.5, 1.5, 0.5), (5.5, 5.5, 0.5), (1.5, 5.5, 0.5)
    t1 = flat_scene([(a, b, c)])
    t2 = flat_scene([(a, c, d)])
    both = flat_scene([(a, b, c), (a, c, d)])
    m1, m2, mb = coverage(oracle, t1), coverage(oracle, t2), coverage(oracle, both)
    assert not np.any(m1 & m2), "a sample on the shared edge was covered twice"
    assert np.array_equal(m1 | m2, mb)
    expected = np.zeros((8, 8), bool)
    expected[1:5, 1:5] = True  # left and top edges in, right and bottom edges out
    assert np.array_equal(mb, expected)


@pytest.mark.parametrize("flip", [False, True])
def test_top_left_rule_both_windings(oracle, flip):
    a, b, c = (1.5, 1.5, 0.5), (5.5, 1.5, 0.5), (1.5, 5.5, 0.5)
    tri = (a, c, b) if flip else (a, b, c)
    m = coverage(oracle, flat_scene([tri]))
    # samples on the top edge y=1.5 (x in [1.5,5.5)) and left edge x=1.5 are in; hypotenuse x+y=7 excluded
    ys, xs = np.nonzero(m)
    expected = {(x, y) for y in range(8) for x in range(8) if x >= 1 and y >= 1 and (x + 0.5) + (y + 0.5) < 7.0}
    assert set(zip(xs.tolist(), ys.tolist())) == expected


def test_fan_has_no_cracks(oracle):
    # 12 triangles around a centre at an odd sub-pixel position: every sample of the disk hit once
    cx, cy = 16.3, 15.7
    pts = [(cx + 12 * math.cos(2 * math.pi * k / 12), cy + 12 * math.sin(2 * math.pi * k / 12)) for k in range(12)]
    tris = [((cx, cy, 0.5), (*pts[k], 0.5), (*pts[(k + 1) % 12], 0.5)) for k in range(12)]
    masks = [coverage(oracle, flat_scene([t], W=32, H=32)) for t in tris]
    total = np.sum(masks, axis=0)
    assert total.max() == 1
    whole = coverage(oracle, flat_scene(tris, W=32, H=32))
    assert np.array_equal(whole, total == 1)


def test_front_face_culling(oracle):
    cw_screen = ((1.5, 1.5, 0.5), (5.5, 1.5, 0.5), (1.5, 5.5, 0.5))  # S > 0: clockwise on screen (y down)
    ccw_screen = (cw_screen[0], cw_screen[2], cw_screen[1])
    # default: front face CLOCKWISE, cull FRONT => clockwise triangles vanish
    assert not coverage(oracle, flat_scene([cw_screen], cull=True)).any()
    assert coverage(oracle, flat_scene([ccw_screen], cull=True)).any()
    # reverse winding: front face COUNTER_CLOCKWISE
    assert coverage(oracle, flat_scene([cw_screen], cull=True, reverse=True)).any()
    assert not coverage(oracle, flat_scene([ccw_screen], cull=True, reverse=True)).any()


def test_greater_or_equal_ties_keep_last_submitted(oracle):
    t = ((0.0, 0.0, 0.4), (8.0, 0.0, 0.4), (0.0, 8.0, 0.4))
    s = one_surface_per_triangle(flat_scene([t, t, t]))
    ids = oracle.raster(s, threads=1)["ids"]
    assert set(np.unique(ids[ids > 0]).tolist()) == {3}


def test_depth_test_nearest_wins_any_order(oracle):
    near = ((0.0, 0.0, 0.9), (8.0, 0.0, 0.9), (0.0, 8.0, 0.9))  # reverse-Z: larger is nearer
    far = ((0.0, 0.0, 0.2), (8.0, 0.0, 0.2), (0.0, 8.0, 0.2))
    for order, winner in (([near, far], 1), ([far, near], 2)):
        r = oracle.raster(one_surface_per_triangle(flat_scene(order)), threads=1)
        ids = r["ids"][r["ids"] > 0]
        assert set(np.unique(ids).tolist()) == {winner}
        assert np.all(r["depth"][r["ids"] > 0] == np.float32(0.9))


def test_near_and_far_clipping(oracle):
    beyond_near = ((0.0, 0.0, 1.5), (8.0, 0.0, 1.2), (0.0, 8.0, 1.1))
    beyond_far = ((0.0, 0.0, -0.5), (8.0, 0.0, -0.2), (0.0, 8.0, -0.1))
    assert not coverage(oracle, flat_scene([beyond_near])).any()
    assert not coverage(oracle, flat_scene([beyond_far])).any()
    crossing = ((0.0, 0.0, 1.5), (8.0, 0.0, 0.5), (0.0, 8.0, 0.5))
    r = oracle.raster(flat_scene([crossing]), threads=1)
    full = coverage(oracle, flat_scene([((0.0, 0.0, 0.9), (8.0, 0.0, 0.5), (0.0, 8.0, 0.5))]))
    m = r["ids"] > 0
    assert 0 < m.sum() < full.sum()
    assert np.all(r["depth"][m] <= 1.0) and np.all(r["depth"][m] > 0.5)


def test_depth_bias_on_sloped_triangle(oracle):
    # shadow pass of a sloped triangle: z(x) = 0.25 + 0.5 * xs / S
    S = 16
    tri = ((0.0, 0.0, 0.25), (16.0, 0.0, 0.75), (0.0, 16.0, 0.25))
    s = flat_scene([tri], W=S, H=S, shadow_size=S)
    s.draw_config["depth_bias_enabled"] = 1
    s.draw_config["depth_bias_constant"] = -21.882
    s.draw_config["depth_bias_clamp"] = -20.937
    s.draw_config["depth_bias_slope_factor"] = -3.0
    biased = oracle.raster(s, threads=1)["shadow"]
    s.draw_config["depth_bias_enabled"] = 0
    plain = oracle.raster(s, threads=1)["shadow"]
    m = plain > 0
    assert m.any()
    slope = 0.5 / S  # depth change per pixel
    r = 2.0 ** (math.frexp(0.75)[1] - 1 - 23)  # e_max of the vertex depths
    o = np.float32(slope * -3.0 + r * -21.882)
    diff = biased[m].astype(np.float64) - plain[m].astype(np.float64)
    assert np.allclose(diff, o, atol=2e-7)


def test_bias_clamp(oracle):
    S = 16
    tri = ((0.0, 0.0, 0.2), (16.0, 0.0, 0.9), (0.0, 16.0, 0.2))
    s = flat_scene([tri], W=S, H=S, shadow_size=S)
    s.draw_config["depth_bias_enabled"] = 1
    s.draw_config["depth_bias_constant"] = 0.0
    s.draw_config["depth_bias_slope_factor"] = -100.0
    s.draw_config["depth_bias_clamp"] = -0.01
    biased = oracle.raster(s, threads=1)["shadow"]
    s.draw_config["depth_bias_enabled"] = 0
    plain = oracle.raster(s, threads=1)["shadow"]
    m = (plain > 0.02)
    assert np.allclose(biased[m], plain[m] - 0.01, atol=1e-6)


def f16(x):
    return np.float32(np.float16(np.float32(x)))


def srgb8(c):
    c = min(max(float(c), 0.0), 1.0)
    c32 = np.float32(c)
    s = c32 * np.float32(12.92) if c32 <= np.float32(0.0031308) else np.float32(1.055) * np.float32(c32) ** np.float32(1 / 2.4) - np.float32(0.055)
    return int(math.floor(np.float32(s) * np.float32(255.0) + np.float32(0.5)))


def test_output_conversion_rgba16f_then_srgb8(oracle):
    col = (0.5, 0.25, 0.00123, 0.7)
    t = ((0.0, 0.0, 0.5), (8.0, 0.0, 0.5), (0.0, 8.0, 0.5))
    out = oracle.render(flat_scene([t], colors=[col]), threads=1)
    px = out["color"][1, 1]
    exp = [srgb8(f16(col[0])), srgb8(f16(col[1])), srgb8(f16(col[2])),
           int(math.floor(f16(col[3]) * np.float32(255) + np.float32(0.5)))]
    assert px.tolist() == exp
    bg = out["color"][7, 7]  # clear colour (0, 0.05, 0.1, 1)
    assert bg.tolist() == [0, srgb8(f16(0.05)), srgb8(f16(0.1)), 255]


def level_colored_texture(size):
    """RGBA8 UNORM-free colour texture whose level l is filled with a distinct grey."""
    levels, flat = [], []
    l, w = 0, size
    while True:
        v = (40 * l + 10) % 256
        flat.append(np.full((w, w, 4), (v, 255 - v, 128, 255), np.uint8).reshape(-1))
        levels.append(v)
        if w == 1:
            break
        w //= 2
        l += 1
    return sc.Texture(size, size, len(levels), sc.IMAGE_NORMAL_MAP, np.concatenate(flat)), levels


@pytest.mark.parametrize("quad_px,expect_level", [(64, 0), (32, 1), (16, 2), (8, 3)])
def test_mip_level_selection(oracle, quad_px, expect_level):
    tex, lv = level_colored_texture(64)
    # a quad of quad_px pixels carrying uv 0..1 over a 64-texel texture => rho = 64/quad_px
    W = H = 64
    x0, x1 = 0.0, float(quad_px)
    tris = [((x0, x0, 0.5), (x1, x0, 0.5), (x1, x1, 0.5)), ((x0, x0, 0.5), (x1, x1, 0.5), (x0, x1, 0.5))]
    uvs = [((0, 0), (1, 0), (1, 1)), ((0, 0), (1, 1), (0, 1))]
    mat = sc.material(color_image=0, sampler=0)
    s = flat_scene(tris, W=W, H=H, material=mat, textures=[tex], uvs=uvs)
    out = oracle.render(s, threads=1)
    # the texture is a normal map (UNORM): output r = sRGB-encode(v/255) of the level's grey
    v = lv[expect_level]
    got = out["color"][quad_px // 2, quad_px // 2]
    assert abs(int(got[0]) - srgb8(f16(np.float32(v) / np.float32(255)))) <= 1


def test_pcf_lit_and_shadowed(oracle):
    # camera: identity; light: z mirrored (z_light = 1 - z), so a surface far from the
    # camera (small z) is near the light and can shadow the receiver the camera sees.
    S = 64
    recv = [((0.0, 0.0, 0.5), (64.0, 0.0, 0.5), (0.0, 64.0, 0.5)), ((64.0, 0.0, 0.5), (64.0, 64.0, 0.5), (0.0, 64.0, 0.5))]
    occ = [((0.0, 0.0, 0.2), (64.0, 0.0, 0.2), (0.0, 64.0, 0.2))]
    mirror = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, -1, 1], [0, 0, 0, 1.0]])
    for tris, lit in ((recv, True), (recv + occ, False)):
        s = flat_scene(tris, W=64, H=64, shadow_size=S, light=True)
        s.scene["shadow_projection_near"] = sc.colmajor(mirror)
        s.scene["shadows_enabled"] = 1
        s.scene["brdf_lighting_enabled"] = 0
        s.scene["ambient_color"] = (0.0, 0.0, 0.0, 1.0)
        s = one_surface_per_triangle(s)
        out = oracle.render(s, threads=1)
        assert out["ids"][5, 5] in (1, 2)  # the camera sees the receiver
        px = out["color"][5, 5]
        if lit:
            assert px[0] > 200
        else:
            assert px[0] == 0
        # outside the occluder's footprint the receiver stays lit
        assert out["color"][60, 60][0] > 200


def test_blended_list_order_and_depth(oracle):
    # opaque red at z 0.5 over the left half; then two blended triangles drawn in order:
    # green (alpha 0.5) at z 0.7 and blue (alpha 0.25) at z 0.3 (behind the opaque: rejected there)
    W = H = 8
    full = ((0.0, 0.0, 0.5), (16.0, 0.0, 0.5), (0.0, 16.0, 0.5))
    g = ((0.0, 0.0, 0.7), (16.0, 0.0, 0.7), (0.0, 16.0, 0.7))
    b = ((0.0, 0.0, 0.3), (16.0, 0.0, 0.3), (0.0, 16.0, 0.3))
    s = flat_scene([full, g, b], W=W, H=H, colors=[(1, 0, 0, 1), (0, 1, 0, 0.5), (0, 0, 1, 0.25)])
    mats = np.concatenate([sc.material(), sc.material(alpha_mode=2), sc.material(alpha_mode=2)])
    s.materials = mats
    s.textures = []
    surf = np.zeros(3, sc.SURFACE_DTYPE)
    surf["index_count"] = 3
    surf["start_index"] = [0, 3, 6]
    surf["material_index"] = [0, 1, 2]
    surf["blended"] = [0, 1, 1]
    s.surfaces = surf
    out = oracle.render(s, threads=1)
    # without textures the material colour factor (1,1,1,a) is the colour; alpha = min(material, vertex)
    px = out["color"][1, 1]
    red = f16(1.0)
    after_g = f16(np.float32(1.0) * np.float32(0.5) + red * np.float32(0.5))  # white-ish (1) over 1
    assert px[3] == int(math.floor(f16(0.5) * np.float32(255) + np.float32(0.5)))  # alpha = last passing blend (0.5)
    assert px[0] == srgb8(after_g)


def test_shadow_cascades_are_scaled_projections(oracle):
    """Cascade k of an n-cascade render is the single-map render with the light's
    clip x and y scaled by 2^-k; fragments inside the finest cascade shade as the
    single-map render with that cascade as its map."""
    from rosy_gb300 import scene as sc

    s = sc.random_triangles(seed=14, triangles=300, width=96, height=64, shadow_size=128, texture_size=32)
    s.scene = s.scene.copy()
    P = s.scene["shadow_projection_near"][0].reshape(4, 4).copy()
    P[:, 0:2] *= 16.0
    s.scene["shadow_projection_near"] = P.reshape(1, 16)
    s.cameras = [s.scene]
    s.draw_config = s.draw_config.copy()
    s.draw_config["shadow_cascades"] = 4
    multi = oracle.raster(s)
    assert multi["shadow"].shape == (4, 128, 128)
    for k in range(4):
        t = sc.Scene(**{f: getattr(s, f) for f in s.__dataclass_fields__})
        t.draw_config = s.draw_config.copy()
        t.draw_config["shadow_cascades"] = 1
        t.scene = s.scene.copy()
        Pk = P.copy()
        Pk[:, 0:2] *= np.float32(2.0 ** -k)
        t.scene["shadow_projection_near"] = Pk.reshape(1, 16)
        single = oracle.raster(t)
        assert np.array_equal(single["shadow"].view(np.uint32), multi["shadow"][k].view(np.uint32)), k
        assert (single["shadow"] > 0).any()
    # coverage grows with the extent
    cov = [(multi["shadow"][k] > 0).mean() for k in range(4)]
    assert cov[0] > cov[1] > cov[2] > cov[3]


def test_msaa_interior_pixels_match_single_sample(oracle):
    """With 4x multisampling a pixel whose four samples all see the triangle its
    centre sees is shaded once at the centre and resolves to exactly the
    single-sample colour ((4 h) / 4 = h in RGBA16F); edge pixels mix."""
    from rosy_gb300 import scene as sc

    s1 = sc.random_triangles(seed=21, triangles=200, width=96, height=64, shadow_size=128, texture_size=32)
    s4 = sc.Scene(**{f: getattr(s1, f) for f in s1.__dataclass_fields__})
    s4.samples = 4
    r1 = oracle.render(s1)
    r4 = oracle.render(s4)
    assert r4["ids"].shape == (4, 64, 96) and r4["depth"].shape == (4, 64, 96)
    same = np.all(r4["ids"] == r1["ids"][None], axis=0)
    assert same.mean() > 0.5 and (~same).any()
    assert np.array_equal(r4["color"][same], r1["color"][same])
    # every sample plane is a valid raster of the same triangles: ids only from the scene
    assert set(np.unique(r4["ids"])) <= set(np.unique(r1["ids"])) | set(range(1, s1.triangle_count + 1))
    # depth and ids agree per sample (0 depth exactly where no triangle)
    assert np.array_equal(r4["depth"] == 0, r4["ids"] == 0)


def test_subpixel_sources_at_a_vertical_edge(oracle):
    """Two triangles meet at x = 4.4 on an 8x8 target. Pixel 3 (centre 3.5) and
    pixel 4 (centre 4.5) straddle the edge: at pixel 4 the points x = 4.25 lie on
    the left triangle, whose bilinear sources there are the left neighbour and the
    left diagonal (bits 1, 3: 0xA); its points x = 4.75 keep every source. At
    pixel 3 the points x = 3.75 keep only own and vertical (bits 0, 2: 0x5).
    Pixels whose neighbourhood shows one triangle keep every source."""
    left = ((-20.0, -20.0, 0.5), (4.4, -20.0, 0.5), (4.4, 40.0, 0.5))
    right = ((4.4, -20.0, 0.5), (30.0, -20.0, 0.5), (4.4, 40.0, 0.5))
    s = flat_scene([left, right])
    ids = oracle.raster(s)["ids"]
    assert (ids[:, :4] == 1).all() and (ids[:, 4:] == 2).all()
    m = oracle.subpixel_sources(s, ids)
    want = np.full((8, 8), 0xFFFF, np.uint16)
    want[:, 3] = 0x5F5F
    want[:, 4] = 0xFAFA
    assert np.array_equal(m, want), [hex(v) for v in m[0]]


def test_subpixel_sources_nearer_triangle_wins(oracle):
    """A small triangle in front (larger depth, reverse-Z) over a background
    triangle, with w = 1 everywhere (so depth, not 1/w, must order them): the
    point (2.25, 2.25) of pixel (2, 2) lies outside the front triangle (which
    starts at 2.3) and takes the back one, shown by the horizontal, vertical and
    diagonal sources (0b1110); the point (2.75, 2.75) lies inside it, and all four
    of its sources show it."""
    back = ((-20.0, -20.0, 0.2), (40.0, -20.0, 0.2), (-20.0, 40.0, 0.2))
    front = ((2.3, 2.3, 0.8), (6.1, 2.3, 0.8), (2.3, 6.1, 0.8))
    s = flat_scene([back, front])
    ids = oracle.raster(s)["ids"]
    m = oracle.subpixel_sources(s, ids)
    assert ids[2, 2] == 2 and ids[1, 1] == 1
    assert m[2, 2] & 0xF == 0b1110
    assert (m[2, 2] >> 12) & 0xF == 0xF
