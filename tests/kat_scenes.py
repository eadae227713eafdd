"""Hand-placed scenes for known-answer tests.

With identity object transforms and an identity view-projection, vertex
positions are clip coordinates (w = 1), so a vertex at framebuffer position
(xs, ys) with depth z is placed at (2*xs/W - 1, 2*ys/H - 1, z).
"""
import numpy as np

from rosy_gb300 import scene as sc


def ndc(xs, ys, W, H):
    return 2.0 * xs / W - 1.0, 2.0 * ys / H - 1.0


def flat_scene(triangles, W=8, H=8, colors=None, shadow_size=16, cull=False, reverse=False,
               light=False, material=None, textures=(), samplers=None, uvs=None, shadow_identity=True):
    """triangles: list of 3 (xs, ys, z) framebuffer-space vertices each."""
    n = len(triangles)
    verts = np.zeros((3 * n, sc.VERTEX_FLOATS), np.float32)
    for t, tri in enumerate(triangles):
        for k, (xs, ys, z) in enumerate(tri):
            x, y = ndc(xs, ys, W, H)
            verts[3 * t + k, 0:3] = (x, y, z)
            verts[3 * t + k, 3:6] = (0, 0, 1)
            verts[3 * t + k, 6:10] = (1, 0, 0, 1)
            c = colors[t] if colors is not None else (1.0, 1.0, 1.0, 1.0)
            verts[3 * t + k, 10:14] = c
            if uvs is not None:
                verts[3 * t + k, 14:16] = uvs[t][k]
    idx = np.arange(3 * n, dtype=np.uint32)
    eye = np.eye(4)
    s = sc.scene_record(eye, eye, (0, 0, 10, 1), eye if shadow_identity else eye, (0, 0, 5), W, H)
    s["view_projection"] = sc.colmajor(eye)
    s["shadow_projection_near"] = sc.colmajor(eye)
    s["light_enabled"] = 1 if light else 0
    s["shadows_enabled"] = 0
    dc = sc.default_draw_config()
    dc["cull_enabled"] = 1 if cull else 0
    dc["reverse_winding_order_enabled"] = 1 if reverse else 0
    dc["depth_bias_enabled"] = 0
    surf = np.zeros(1, sc.SURFACE_DTYPE)
    surf["index_count"] = 3 * n
    surf["material_index"] = 0 if material is not None else sc.U32_MAX
    mats = material if material is not None else np.zeros(0, sc.MATERIAL_DTYPE)
    return sc.Scene(name="kat", width=W, height=H, shadow_size=shadow_size, vertices=verts, indices=idx,
                    meshes=[(0, 3 * n, 0, 3 * n)], objects=sc.object_record(eye)[None, :], surfaces=surf,
                    materials=mats, textures=list(textures),
                    samplers=samplers if samplers is not None else sc.linear_sampler(),
                    scene=s, draw_config=dc, cameras=[s])


def one_surface_per_triangle(s):
    """Same scene with one draw per triangle (submission order = triangle order)."""
    n = len(s.indices) // 3
    surf = np.zeros(n, sc.SURFACE_DTYPE)
    surf["index_count"] = 3
    surf["start_index"] = np.arange(n) * 3
    surf["material_index"] = s.surfaces["material_index"][0]
    s.surfaces = surf
    return s


def random_texture(rng, width, height, image_type):
    """A texture of any extent (odd and non-power-of-two levels included) with a
    full mip chain of seeded random texels; every level is max(1, size >> l)."""
    levels = 1
    while max(width, height) >> levels:
        levels += 1
    parts = []
    for l in range(levels):
        w, h = max(1, width >> l), max(1, height >> l)
        parts.append(rng.integers(0, 256, (h, w, 4), dtype=np.uint8).reshape(-1))
    return sc.Texture(width, height, levels, image_type, np.concatenate(parts))


def sampler(min_filter, mag_filter, wrap_s, wrap_t):
    s = np.zeros(1, sc.SAMPLER_DTYPE)
    s["min_filter"], s["mag_filter"], s["wrap_s"], s["wrap_t"] = min_filter, mag_filter, wrap_s, wrap_t
    return s


# (min filter, mag filter, wrap s, wrap t) codes of the asset format: filters 0-2
# nearest and 3-5 linear, wraps 0 clamp, 1 mirrored repeat, 2 repeat
# (src/Engine/Graphics.cpp:250-278); 6 and 9 are out of the documented range
# and fall to the switches' default cases (linear, repeat)
ZOO_SAMPLERS = [(5, 3, 2, 2), (0, 0, 0, 0), (2, 3, 1, 1), (4, 1, 0, 2), (5, 5, 2, 1), (1, 4, 1, 0), (3, 2, 9, 6),
                (6, 0, 0, 1)]


def material_zoo(seed=0, triangles=3000, width=320, height=200, shadow_size=256, texture_size=64):
    """Random triangles split into draws that reach every material and sampler
    branch of the fragment program (src/shaders/basic.slang:138-344):

    * colour / normal / metal-roughness textures; a mixmap beside a metallic
      texture (the mixmap wins); a mixmap alone; a metallic texture absent (its
      sample reads zeros); a material with no textures; a draw with no material;
    * every filter and wrap code (ZOO_SAMPLERS), the default sampler (linear,
      nearest mip, repeat: src/Engine/Graphics.cpp:3421-3438) through an
      out-of-range sampler index, square power-of-two and odd-sized textures;
    * per-triangle uv scales from 1/32 to 16 and offsets outside [0, 1], so each
      draw meets magnification, minification and the wrap modes."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = sc.random_triangles(seed=seed, triangles=triangles, width=width, height=height, shadow_size=shadow_size,
                            texture_size=texture_size)
    t = len(s.indices) // 3
    uv = s.vertices[:, 14:16].reshape(t, 3, 2).astype(np.float64)
    scale = np.exp(rng.uniform(np.log(1 / 32), np.log(16), (t, 1, 1)))
    shift = rng.uniform(-3.0, 3.0, (t, 1, 2))
    s.vertices[:, 14:16] = (uv * scale + shift).reshape(-1, 2).astype(np.float32)
    n = texture_size
    tex = [sc.make_texture(rng, n, sc.IMAGE_COLOR), sc.make_texture(rng, n, sc.IMAGE_NORMAL_MAP),
           sc.make_texture(rng, n, sc.IMAGE_METALLIC_ROUGHNESS), sc.make_texture(rng, n, sc.IMAGE_MIXMAP),
           random_texture(rng, 37, 23, sc.IMAGE_COLOR), random_texture(rng, 29, 50, sc.IMAGE_MIXMAP),
           random_texture(rng, 45, 45, sc.IMAGE_NORMAL_MAP)]
    C, N, M, X, C_ODD, X_ODD, N_ODD = range(7)
    U = sc.U32_MAX
    mats = [
        sc.material(color_image=C, normal_image=N, metallic_image=M, sampler=0),
        sc.material(color_image=C, metallic_image=M, mixmap_image=X, sampler=1),
        sc.material(color_image=C_ODD, mixmap_image=X, sampler=2),
        sc.material(color_image=C_ODD, normal_image=N_ODD, sampler=3),
        sc.material(color_image=C, metallic_image=M, sampler=99),
        sc.material(color_image=C_ODD, normal_image=N, mixmap_image=X_ODD, sampler=4),
        sc.material(base_color=(0.8, 0.45, 0.2, 1.0)),
        sc.material(color_image=C, normal_image=N_ODD, metallic_image=M, sampler=5),
        sc.material(color_image=C_ODD, mixmap_image=X_ODD, sampler=6),
        sc.material(color_image=C, normal_image=N, metallic_image=M, sampler=7),
    ]
    # one sampler slot per material may differ from the others: the normal map of
    # material 0 uses the default sampler, the mixmap of material 1 the last code
    mats[0]["normal_sampler_index"] = 200
    mats[1]["mixmap_sampler_index"] = 7
    for m, f in zip(mats, rng.uniform(0.3, 1.0, (len(mats), 2))):
        m["metallic_factor"], m["roughness_factor"] = f
    draws = len(mats) + 1  # the last draw has no material
    bounds = np.linspace(0, t, draws + 1).astype(int)
    surf = np.zeros(draws, sc.SURFACE_DTYPE)
    surf["start_index"] = bounds[:-1] * 3
    surf["index_count"] = np.diff(bounds) * 3
    surf["material_index"] = list(range(len(mats))) + [U]
    s.surfaces = surf
    s.materials = np.concatenate(mats)
    s.textures = tex
    s.samplers = np.concatenate([sampler(*z) for z in ZOO_SAMPLERS])
    s.name = f"material_zoo_s{seed}_{width}x{height}"
    return s
