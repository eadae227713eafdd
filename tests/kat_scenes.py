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
