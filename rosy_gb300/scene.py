"""Seeded synthetic scenes with the reference's data layouts.

Rosy ships no assets in its source tree (the level file points at .rsy files
that are not there, src/Engine/level1.json:1-40), so every input here is
generated from a seed with numpy's PCG64 generator:

* vertices in the 64-byte ``rosy_asset::position`` layout (src/Asset/Asset.h:92-99),
* u32 mesh-local indices, concatenated per mesh (src/Engine/Graphics.cpp:4310-4334),
* per-object transforms built like ``node::populate_graph``
  (src/Engine/Node.cpp:96-118, 233-249): world = T * R(yaw about -y) * S,
  to-object = inverse(world), normal = transpose(inverse(mat3(world))),
* the camera of ``camera::update`` (src/Engine/Camera.cpp:62-98, 258-279):
  reverse-Z projection with the Vulkan y/z flip, view = inverse(T * R),
  camera_position.w left at 0 as the reference leaves it,
* the sun and its orthographic shadow projection of src/Engine/Level.cpp:455-527,
* render defaults of src/Engine/Level.cpp:1240-1264.

Textures are RGBA8 value noise with full box-filtered mip chains. Matrices are
column-major float32 (glm's layout), flattened.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

U32_MAX = 0xFFFFFFFF

# --- record layouts (must match include/rosy_gb300.h) ---------------------------

VERTEX_FLOATS = 16  # rz_vertex: pos3 nrm3 tan4 col4 uv2 = 64 B
OBJECT_FLOATS = 41  # rz_object: 16 + 16 + 9 floats = 164 B

MATERIAL_DTYPE = np.dtype([
    ("base_color_factor", "<f4", 4),
    ("metallic_factor", "<f4"),
    ("roughness_factor", "<f4"),
    ("alpha_cutoff", "<f4"),
    ("alpha_mode", "<u4"),
    ("double_sided", "<u4"),
    ("color_image_index", "<u4"),
    ("color_sampler_index", "<u4"),
    ("normal_image_index", "<u4"),
    ("normal_sampler_index", "<u4"),
    ("metallic_image_index", "<u4"),
    ("metallic_sampler_index", "<u4"),
    ("mixmap_image_index", "<u4"),
    ("mixmap_sampler_index", "<u4"),
])
assert MATERIAL_DTYPE.itemsize == 68

SAMPLER_DTYPE = np.dtype([("min_filter", "<u2"), ("mag_filter", "<u2"),
                          ("wrap_s", "<u2"), ("wrap_t", "<u2")])

SURFACE_DTYPE = np.dtype([
    ("mesh_index", "<u4"), ("graphic_objects_offset", "<u4"),
    ("graphics_object_index", "<u4"), ("material_index", "<u4"),
    ("index_count", "<u4"), ("start_index", "<u4"), ("blended", "<u4"),
])

# rz_debug_object: the debug-line overlay (src/Engine/Types.h:81-98)
DEBUG_OBJECT_DTYPE = np.dtype([("type", "<u4"), ("flags", "<u4"), ("transform", "<f4", 16), ("color", "<f4", 4)])
DEBUG_LINE, DEBUG_CIRCLE, DEBUG_CROSS = 0, 1, 2
DEBUG_SCREEN_SPACE, DEBUG_VIEW_SPACE, DEBUG_TRANSFORM_IS_POINTS = 1, 2, 4


def debug_object(kind: int, transform, color, flags: int = 0) -> np.ndarray:
    """One overlay object; `transform` is a row-major math matrix (stored column-major)."""
    o = np.zeros(1, DEBUG_OBJECT_DTYPE)
    o["type"] = kind
    o["flags"] = flags
    o["transform"] = colmajor(transform)
    o["color"] = color
    return o


SCENE_DTYPE = np.dtype([
    ("view", "<f4", 16), ("proj", "<f4", 16), ("view_projection", "<f4", 16),
    ("shadow_projection_near", "<f4", 16),
    ("sun_position", "<f4", 4), ("camera_position", "<f4", 4),
    ("ambient_color", "<f4", 4), ("sunlight_color", "<f4", 4),
    ("flip_lights", "<u4", 4), ("flip_tangents", "<u4", 4),
    ("draw_extent", "<f4", 2), ("light_intensity", "<f4"),
    ("csm_index_sampler", "<u4"), ("csm_index_near", "<u4"),
    ("fragment_output", "<u4"), ("light_enabled", "<u4"),
    ("tangent_space_enabled", "<u4"), ("shadows_enabled", "<u4"),
    ("normal_maps_enabled", "<u4"), ("inverse_bnt", "<u4"),
    ("ignore_asset_tangent_sign", "<u4"), ("ensure_orthogonal_bitangent", "<u4"),
    ("brdf_lighting_enabled", "<u4"),
])
assert SCENE_DTYPE.itemsize == 408

DRAW_CONFIG_DTYPE = np.dtype([
    ("cull_enabled", "<u4"), ("reverse_winding_order_enabled", "<u4"),
    ("depth_bias_enabled", "<u4"), ("depth_bias_constant", "<f4"),
    ("depth_bias_clamp", "<f4"), ("depth_bias_slope_factor", "<f4"),
    ("pcf_mode", "<u4"), ("shadow_cascades", "<u4"),
])

IMAGE_COLOR, IMAGE_NORMAL_MAP, IMAGE_METALLIC_ROUGHNESS, IMAGE_MIXMAP = 0, 1, 2, 3
PCF_5TAP, PCF_3X3 = 0, 1

# Render defaults, src/Engine/Level.cpp:1240-1264.
SUN_DISTANCE = 23.776
ORTHOGRAPHIC_DEPTH = 76.838
CASCADE_LEVEL = 36.0
DEPTH_BIAS_CONSTANT = -21.882
DEPTH_BIAS_CLAMP = -20.937
DEPTH_BIAS_SLOPE = -3.0
LIGHT_INTENSITY = 5.2
AMBIENT_LIGHT = 0.01
NEAR, FAR = 0.1, 1000.0  # src/Engine/Camera.h:27-28


@dataclass
class Texture:
    width: int
    height: int
    levels: int
    image_type: int
    texels: np.ndarray  # uint8, all levels concatenated (RGBA8, or BC7 blocks when format is 1)
    format: int = 0     # 0 RGBA8, 1 BC7 blocks

    def level_offset(self, level: int) -> int:
        off = 0
        for l in range(level):
            off += max(1, self.width >> l) * max(1, self.height >> l) * 4
        return off


@dataclass
class Scene:
    name: str
    width: int
    height: int
    shadow_size: int
    vertices: np.ndarray  # (V, 16) float32, all meshes concatenated
    indices: np.ndarray  # (I,) uint32, mesh-local
    meshes: list  # [(vertex_offset, vertex_count, index_offset, index_count)]
    objects: np.ndarray  # (O, 41) float32
    surfaces: np.ndarray  # SURFACE_DTYPE
    materials: np.ndarray  # MATERIAL_DTYPE
    textures: list  # [Texture]
    samplers: np.ndarray  # SAMPLER_DTYPE
    scene: np.ndarray  # SCENE_DTYPE, shape (1,)
    draw_config: np.ndarray  # DRAW_CONFIG_DTYPE, shape (1,)
    cameras: list = field(default_factory=list)  # extra SCENE_DTYPE records (one per frame)
    samples: int = 1  # camera-pass samples per pixel (1, or 4: the reference's 4x MSAA)
    debug_objects: np.ndarray | None = None  # DEBUG_OBJECT_DTYPE: the debug-line overlay, or None

    @property
    def triangle_count(self) -> int:
        return int(self.surfaces["index_count"].sum() // 3)

    def with_camera(self, i: int) -> "Scene":
        """The same scene with the scene constants of camera frame i."""
        s = Scene(**{k: getattr(self, k) for k in self.__dataclass_fields__})
        s.scene = self.cameras[i % len(self.cameras)]
        return s


# --- matrix helpers (float64 math, column-major float32 output) -----------------

def _translate(t):
    m = np.eye(4)
    m[:3, 3] = t
    return m


def _scale(s):
    return np.diag([s, s, s, 1.0])


def _rot_x(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1, 0, 0, 0], [0, c, -s, 0], [0, s, c, 0], [0, 0, 0, 1.0]])


def _rot_y(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1.0]])


def colmajor(m) -> np.ndarray:
    """Row-major math matrix -> glm column-major flat float32."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.float64).T.reshape(-1)).astype(np.float32)


def projection(aspect: float, fov_rad: float, n: float = NEAR, f: float = FAR):
    """camera get_projection, src/Engine/Camera.cpp:62-83 (reverse-Z, y/z flip)."""
    h = 1.0 / math.tan(fov_rad * 0.5)
    w = h / aspect
    a = -n / (f - n)
    b = (n * f) / (f - n)
    m = np.array([[w, 0, 0, 0], [0, h, 0, 0], [0, 0, a, b], [0, 0, 1, 0]], dtype=np.float64)
    ndc = np.diag([1.0, -1.0, -1.0, 1.0])
    return m @ ndc


def camera_look_at_origin(position, target=(0.0, 0.0, 0.0)):
    """View matrix of src/Engine/Camera.cpp:85-98 with yaw/pitch chosen so the
    camera's -z axis points from `position` to `target`."""
    d = np.asarray(position, np.float64) - np.asarray(target, np.float64)
    d /= np.linalg.norm(d)
    pitch = math.asin(max(-1.0, min(1.0, d[1])))
    yaw = math.atan2(d[0], d[2])
    rot = _rot_y(yaw) @ _rot_x(-pitch)  # yaw about +y, pitch about -x
    return np.linalg.inv(_translate(position) @ rot)


def sun_matrices(direction):
    """Sun position and shadow projection of src/Engine/Level.cpp:455-527 for a
    unit direction pointing from the origin towards the sun."""
    u = np.asarray(direction, np.float64)
    u = u / np.linalg.norm(u)
    pitch = math.asin(max(-1.0, min(1.0, -u[1])))
    yaw = math.atan2(u[0], -u[2])
    # light_line_rot = R(yaw about -y) * R(-pitch about x)
    line_rot = _rot_y(-yaw) @ _rot_x(-pitch)
    sun_position = line_rot @ np.array([0.0, 0.0, -SUN_DISTANCE, 1.0])
    light_view = line_rot @ _translate([0.0, 0.0, SUN_DISTANCE])
    lp = np.diag([-2.0 / CASCADE_LEVEL, -2.0 / CASCADE_LEVEL, -1.0 / ORTHOGRAPHIC_DEPTH, 1.0])
    shadow_projection_near = lp @ np.linalg.inv(light_view)
    return sun_position, shadow_projection_near


def object_record(world) -> np.ndarray:
    """graphic_object_data of src/Engine/Node.cpp:233-249."""
    world = np.asarray(world, np.float64)
    rec = np.zeros(OBJECT_FLOATS, np.float32)
    rec[0:16] = colmajor(world)
    rec[16:32] = colmajor(np.linalg.inv(world))
    nrm = np.linalg.inv(world[:3, :3]).T
    rec[32:41] = np.ascontiguousarray(nrm.T.reshape(-1)).astype(np.float32)
    return rec


def node_world(translate, scale, yaw):
    """node world transform T * R(yaw about -y) * S (src/Engine/Node.cpp:96-103)."""
    return _translate(translate) @ _rot_y(-yaw) @ _scale(scale)


def scene_record(view, proj, sun_position, shadow_projection_near, cam_pos, width, height,
                 **overrides) -> np.ndarray:
    """gpu_scene_data as packed by graphics_device::update (src/Engine/Graphics.cpp:6016-6061)
    with the defaults of src/Engine/Level.cpp:1240-1264."""
    s = np.zeros(1, SCENE_DTYPE)
    s["view"] = colmajor(view)
    s["proj"] = colmajor(proj)
    # vp = proj * view is formed in float32 by glm on the host (Camera.cpp:272)
    p32 = colmajor(proj).reshape(4, 4).T.astype(np.float32)
    v32 = colmajor(view).reshape(4, 4).T.astype(np.float32)
    s["view_projection"] = np.ascontiguousarray((p32 @ v32).T.reshape(-1)).astype(np.float32)
    s["shadow_projection_near"] = colmajor(shadow_projection_near)
    s["sun_position"] = np.asarray(sun_position, np.float32)
    s["camera_position"] = np.array([cam_pos[0], cam_pos[1], cam_pos[2], 0.0], np.float32)
    s["ambient_color"] = np.array([AMBIENT_LIGHT, AMBIENT_LIGHT, AMBIENT_LIGHT, 1.0], np.float32)
    s["sunlight_color"] = np.array([1.0, 1.0, 1.0, 1.0], np.float32)
    s["flip_lights"] = np.array([0, 0, 0, 1], np.uint32)
    s["flip_tangents"] = np.array([0, 0, 0, 0], np.uint32)
    s["draw_extent"] = np.array([width, height], np.float32)
    s["light_intensity"] = LIGHT_INTENSITY
    s["fragment_output"] = 0
    s["light_enabled"] = 1
    s["tangent_space_enabled"] = 1
    s["shadows_enabled"] = 1
    s["normal_maps_enabled"] = 1
    s["brdf_lighting_enabled"] = 1
    for k, v in overrides.items():
        s[k] = v
    return s


def default_draw_config(pcf_mode: int = PCF_5TAP) -> np.ndarray:
    d = np.zeros(1, DRAW_CONFIG_DTYPE)
    d["cull_enabled"] = 1
    d["reverse_winding_order_enabled"] = 0
    d["depth_bias_enabled"] = 1
    d["depth_bias_constant"] = DEPTH_BIAS_CONSTANT
    d["depth_bias_clamp"] = DEPTH_BIAS_CLAMP
    d["depth_bias_slope_factor"] = DEPTH_BIAS_SLOPE
    d["pcf_mode"] = pcf_mode
    return d


# --- textures -------------------------------------------------------------------

def value_noise(rng, size: int, cells: int, channels: int, octaves: int = 3) -> np.ndarray:
    """Tileable value noise in [0,1], shape (size, size, channels), float32."""
    out = np.zeros((size, size, channels), np.float32)
    amp, total = 1.0, 0.0
    c = cells
    for _ in range(octaves):
        c = max(1, min(c, size))
        lattice = rng.random((channels, c, c), dtype=np.float32)
        x = (np.arange(size, dtype=np.float32) + 0.5) * (c / size)
        i0 = np.floor(x).astype(np.int64)
        f = x - i0
        f = f * f * (3.0 - 2.0 * f)
        i0 %= c
        i1 = (i0 + 1) % c
        for ch in range(channels):
            L = lattice[ch]
            a = L[i0][:, i0] * (1 - f)[None, :] + L[i0][:, i1] * f[None, :]
            b = L[i1][:, i0] * (1 - f)[None, :] + L[i1][:, i1] * f[None, :]
            out[:, :, ch] += amp * (a * (1 - f)[:, None] + b * f[:, None])
        total += amp
        amp *= 0.5
        c *= 2
    return out / total


def value_noise_separable(rng, size: int, cells: int, channels: int, octaves: int = 3) -> np.ndarray:
    """The same tileable smoothstep value noise as value_noise, evaluated as
    W @ lattice @ W^T per octave (W: size x cells interpolation weights), which
    is fast for large textures; values agree with value_noise to float rounding."""
    out = np.zeros((channels, size, size), np.float32)
    amp, total = 1.0, 0.0
    c = cells
    for _ in range(octaves):
        c = max(1, min(c, size))
        lattice = rng.random((channels, c, c), dtype=np.float32)
        x = (np.arange(size, dtype=np.float32) + 0.5) * (c / size)
        i0 = np.floor(x).astype(np.int64)
        f = x - i0
        f = f * f * (3.0 - 2.0 * f)
        i0 %= c
        i1 = (i0 + 1) % c
        Wm = np.zeros((size, c), np.float32)
        np.add.at(Wm, (np.arange(size), i0), 1.0 - f)
        np.add.at(Wm, (np.arange(size), i1), f)
        out += amp * (Wm[None] @ lattice @ Wm.T[None])
        total += amp
        amp *= 0.5
        c *= 2
    return np.ascontiguousarray((out / total).transpose(1, 2, 0))


def build_mips(level0: np.ndarray) -> tuple[np.ndarray, int]:
    """Full box-filtered mip chain of an (h, w, 4) uint8 image (power-of-two sizes)."""
    h, w, _ = level0.shape
    levels = [level0]
    cur = level0.astype(np.float32)
    while cur.shape[0] > 1 or cur.shape[1] > 1:
        hh, ww = max(1, cur.shape[0] // 2), max(1, cur.shape[1] // 2)
        if cur.shape[0] > 1 and cur.shape[1] > 1:
            nxt = 0.25 * (cur[0::2, 0::2] + cur[1::2, 0::2] + cur[0::2, 1::2] + cur[1::2, 1::2])
        elif cur.shape[0] > 1:
            nxt = 0.5 * (cur[0::2] + cur[1::2])
        else:
            nxt = 0.5 * (cur[:, 0::2] + cur[:, 1::2])
        nxt = nxt.reshape(hh, ww, 4)
        levels.append(np.clip(np.floor(nxt + 0.5), 0, 255).astype(np.uint8))
        cur = levels[-1].astype(np.float32)
    flat = np.concatenate([l.reshape(-1) for l in levels])
    return flat, len(levels)


def make_texture(rng, size: int, image_type: int, cells: int = 16, separable: bool = False) -> Texture:
    noise = value_noise_separable if separable else value_noise
    if image_type == IMAGE_NORMAL_MAP:
        n = noise(rng, size, cells, 2) * 0.8 - 0.4
        nz = np.sqrt(np.maximum(0.0, 1.0 - n[..., 0] ** 2 - n[..., 1] ** 2))
        rgb = np.stack([n[..., 0], n[..., 1], nz], -1) * 0.5 + 0.5
        a = np.ones(rgb.shape[:2] + (1,), np.float32)
        img = np.concatenate([rgb, a], -1)
    elif image_type == IMAGE_METALLIC_ROUGHNESS or image_type == IMAGE_MIXMAP:
        n = noise(rng, size, cells, 2)
        img = np.stack([np.ones_like(n[..., 0]), 0.15 + 0.85 * n[..., 0],
                        np.clip(n[..., 1] * 1.6 - 0.5, 0, 1), np.ones_like(n[..., 0])], -1)
    else:
        n = noise(rng, size, cells, 3)
        rgb = 0.1 + 0.85 * n
        img = np.concatenate([rgb, np.ones(rgb.shape[:2] + (1,), np.float32)], -1)
    img8 = np.clip(np.floor(img * 255.0 + 0.5), 0, 255).astype(np.uint8)
    flat, levels = build_mips(img8)
    return Texture(size, size, levels, image_type, flat)


def linear_sampler(wrap: int = 2) -> np.ndarray:
    s = np.zeros(1, SAMPLER_DTYPE)
    s["min_filter"] = 5  # LinearMipMapLinear (src/Packager/Gltf.cpp:31-48)
    s["mag_filter"] = 3  # Linear
    s["wrap_s"] = wrap
    s["wrap_t"] = wrap
    return s


def material(color_image=U32_MAX, normal_image=U32_MAX, metallic_image=U32_MAX,
             mixmap_image=U32_MAX, sampler=0, alpha_mode=0, alpha_cutoff=0.0,
             base_color=(1.0, 1.0, 1.0, 1.0)) -> np.ndarray:
    m = np.zeros(1, MATERIAL_DTYPE)
    m["base_color_factor"] = base_color
    m["metallic_factor"] = 1.0
    m["roughness_factor"] = 1.0
    m["alpha_cutoff"] = alpha_cutoff
    m["alpha_mode"] = alpha_mode
    for name, idx in (("color", color_image), ("normal", normal_image),
                      ("metallic", metallic_image), ("mixmap", mixmap_image)):
        m[f"{name}_image_index"] = idx
        m[f"{name}_sampler_index"] = sampler if idx != U32_MAX else U32_MAX
    return m


def _unit(rng, n):
    v = rng.standard_normal((n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _tangents(rng, normals):
    t = rng.standard_normal(normals.shape)
    t -= normals * np.sum(t * normals, axis=1, keepdims=True)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    w = np.where(rng.random(len(normals)) < 0.5, -1.0, 1.0)
    return np.concatenate([t, w[:, None]], 1)


# --- config 1: one mesh of independent random triangles ---------------------------

def random_triangles(seed: int = 0, triangles: int = 4096, width: int = 640, height: int = 360,
                     shadow_size: int = 1024, texture_size: int = 256, fov_deg: float = 60.0,
                     pcf_mode: int = PCF_5TAP) -> Scene:
    """One indexed mesh of independent triangles with vertices uniform in [-1,1]^3,
    one value-noise albedo texture with a full mip chain, a seeded sun direction
    and a camera on the radius-3 sphere looking at the origin."""
    rng = np.random.Generator(np.random.PCG64(seed))
    V = triangles * 3
    pos = rng.uniform(-1.0, 1.0, (V, 3))
    nrm = _unit(rng, V)
    tan = _tangents(rng, nrm)
    uv = rng.random((V, 2))
    verts = np.zeros((V, VERTEX_FLOATS), np.float32)
    verts[:, 0:3] = pos
    verts[:, 3:6] = nrm
    verts[:, 6:10] = tan
    verts[:, 10:14] = 1.0
    verts[:, 14:16] = uv
    idx = np.arange(V, dtype=np.uint32)
    tex = make_texture(rng, texture_size, IMAGE_COLOR, cells=16)
    sun_dir = _unit(rng, 1)[0]
    sun_dir[1] = abs(sun_dir[1]) + 0.3
    cam_dir = _unit(rng, 1)[0]
    cam_pos = 3.0 * cam_dir
    sun_position, spn = sun_matrices(sun_dir)
    view = camera_look_at_origin(cam_pos)
    proj = projection(width / height, math.radians(fov_deg))
    sc = scene_record(view, proj, sun_position, spn, cam_pos, width, height)
    surf = np.zeros(1, SURFACE_DTYPE)
    surf["index_count"] = V
    return Scene(
        name=f"random_triangles_s{seed}_t{triangles}_{width}x{height}",
        width=width, height=height, shadow_size=shadow_size,
        vertices=verts, indices=idx, meshes=[(0, V, 0, V)],
        objects=object_record(np.eye(4))[None, :],
        surfaces=surf,
        materials=material(color_image=0, sampler=0),
        textures=[tex], samplers=linear_sampler(),
        scene=sc, draw_config=default_draw_config(pcf_mode), cameras=[sc])


def _rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    w, x, y, z = q / np.linalg.norm(q)
    r = np.eye(4)
    r[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                 [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                 [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
    return r


def random_debug_objects(seed: int, n: int, extent: float = 2.5) -> np.ndarray:
    """n seeded overlay objects of every kind around a scene of half-size ~1 seen from
    distance 3: world-space lines (some crossing the near plane), crosses and circles,
    screen- and view-space lines and circles, "transform is points" lines, and flags
    that match none of the spaces (3, 5: world space, as the shader's equality tests give)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n):
        kind = i % 8
        color = (*rng.random(3), 1.0)
        if kind in (0, 1):  # world-space line / cross between two random points
            a, b = rng.uniform(-extent, extent, 3), rng.uniform(-extent, extent, 3)
            t = np.eye(4)
            t[:3, 2] = b - a
            t[:3, 3] = a
            out.append(debug_object(DEBUG_LINE if kind == 0 else DEBUG_CROSS, t, color, int(rng.choice([0, 3, 5]))))
        elif kind == 2:  # world-space circle
            t = _translate(rng.uniform(-1.5, 1.5, 3)) @ _rotation(rng) @ _scale(rng.uniform(0.2, 1.5))
            out.append(debug_object(DEBUG_CIRCLE, t, color))
        elif kind in (3, 4):  # screen-space line / circle
            t = _translate((*rng.uniform(-1, 1, 2), 0.0)) @ _rotation(rng) @ _scale(rng.uniform(0.05, 0.6))
            out.append(debug_object(DEBUG_LINE if kind == 3 else DEBUG_CIRCLE, t, color, DEBUG_SCREEN_SPACE))
        elif kind in (5, 6):  # view-space line / circle
            t = _translate((*rng.uniform(-1, 1, 2), -rng.uniform(1, 5))) @ _rotation(rng) @ _scale(rng.uniform(0.1, 1))
            out.append(debug_object(DEBUG_LINE if kind == 5 else DEBUG_CIRCLE, t, color, DEBUG_VIEW_SPACE))
        else:  # points: columns 0 and 1 are the ends
            pts = np.ones((4, 4))
            pts[:3, 0] = rng.uniform(-extent, extent, 3)
            pts[:3, 1] = rng.uniform(-extent, extent, 3)
            out.append(debug_object(DEBUG_LINE, pts, color, DEBUG_TRANSFORM_IS_POINTS))
    return np.concatenate(out)


# --- config 2: many tessellated meshes, materials, camera spline -------------------

def uv_sphere(rings: int, segments: int, uv_repeat: float = 4.0):
    """A UV sphere of radius 1 with 2*rings*segments triangles."""
    r = np.arange(rings + 1) / rings
    s = np.arange(segments + 1) / segments
    th = r[:, None] * math.pi
    ph = s[None, :] * 2.0 * math.pi
    x = np.sin(th) * np.cos(ph)
    y = np.cos(th) * np.ones_like(ph)
    z = np.sin(th) * np.sin(ph)
    pos = np.stack([x, y, z], -1).reshape(-1, 3)
    nrm = pos.copy()
    tx = -np.sin(ph) * np.ones_like(th)
    tz = np.cos(ph) * np.ones_like(th)
    tan = np.stack([tx, np.zeros_like(tx), tz, np.ones_like(tx)], -1).reshape(-1, 4)
    uu = np.broadcast_to(s[None, :], (rings + 1, segments + 1)) * uv_repeat * 2
    vv = np.broadcast_to(r[:, None], (rings + 1, segments + 1)) * uv_repeat
    uv = np.stack([uu, vv], -1).reshape(-1, 2)
    idx = []
    for i in range(rings):
        for j in range(segments):
            a = i * (segments + 1) + j
            b = a + segments + 1
            # counter-clockwise seen from outside: kept by the reference's cull-front/CW-front state
            idx += [a, a + 1, b, a + 1, b + 1, b]
    return pos, nrm, tan, uv, np.asarray(idx, np.uint32)


def catmull_rom(p0, p1, p2, p3, t):
    t2, t3 = t * t, t * t * t
    return 0.5 * ((2 * p1) + (-p0 + p2) * t + (2 * p0 - 5 * p1 + 4 * p2 - p3) * t2
                  + (-p0 + 3 * p1 - 3 * p2 + p3) * t3)


def scene_scale(seed: int = 0, meshes: int = 64, triangles_per_mesh: int = 4096, materials: int = 32,
                texture_size: int = 1024, width: int = 1920, height: int = 1080, shadow_size: int = 4096,
                frames: int = 8, fov_deg: float = 60.0, median_area_px: float = 4.0, sigma: float = 1.5,
                pcf_mode: int = PCF_3X3, texture_workers: int = 0) -> Scene:
    """Meshes (UV spheres) whose per-mesh triangle screen area at the first camera
    is log-normal(median, sigma); each material has albedo (sRGB), normal (UNORM)
    and metal-roughness (sRGB) textures with full mips; per-draw material IDs;
    camera frames along a seeded Catmull-Rom spline. With texture_workers > 0 the
    textures come from per-texture seeds on that many threads with the separable
    noise (a different, faster stream of the same kind of noise)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    segs = 64
    rings = max(1, triangles_per_mesh // (2 * segs))
    if 2 * rings * segs != triangles_per_mesh:
        segs = max(1, triangles_per_mesh // 2)
        rings = 1
    spos, snrm, stan, suv, sidx = uv_sphere(rings, segs)
    nv = len(spos)

    # camera spline on a jittered ring around the origin
    ctrl = []
    for k in range(4):
        ang = 2 * math.pi * (k / 4.0) * 0.35 + rng.uniform(-0.1, 0.1)
        rad = 24.0 + rng.uniform(-2, 2)
        ctrl.append(np.array([rad * math.sin(ang), 5.0 + rng.uniform(-1.5, 1.5), rad * math.cos(ang)]))
    cam_positions = [catmull_rom(*ctrl, t) for t in np.linspace(0.0, 1.0, frames, endpoint=False)]
    cam0 = cam_positions[0]
    f_px = (height * 0.5) / math.tan(math.radians(fov_deg) * 0.5)

    # object placement inside the shadow cascade (|x|,|z| < 16) and in front of camera 0
    verts = np.zeros((meshes * nv, VERTEX_FLOATS), np.float32)
    idx = np.zeros(meshes * len(sidx), np.uint32)
    mesh_list, objects = [], []
    areas = np.exp(np.log(median_area_px) + sigma * rng.standard_normal(meshes))
    for m in range(meshes):
        center = np.array([rng.uniform(-14, 14), rng.uniform(-1.0, 4.0), rng.uniform(-14, 14)])
        d = float(np.linalg.norm(center - cam0))
        # mean triangle area of the unit sphere mesh, visible-hemisphere foreshortening ~0.5
        tri_area = 4.0 * math.pi / triangles_per_mesh
        r = math.sqrt(areas[m] * d * d / (tri_area * f_px * f_px * 0.5))
        r = float(min(r, 0.45 * max(d - 1.0, 0.2), 6.0))
        squash = np.array([1.0, rng.uniform(0.6, 1.2), 1.0])
        p = spos * squash
        n = snrm / squash
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        v0 = m * nv
        verts[v0:v0 + nv, 0:3] = p
        verts[v0:v0 + nv, 3:6] = n
        verts[v0:v0 + nv, 6:10] = stan
        verts[v0:v0 + nv, 10:14] = 1.0
        verts[v0:v0 + nv, 14:16] = suv
        i0 = m * len(sidx)
        idx[i0:i0 + len(sidx)] = sidx
        mesh_list.append((v0, nv, i0, len(sidx)))
        objects.append(object_record(node_world(center, r, rng.uniform(0, 2 * math.pi))))
    textures, mats = [], []
    kinds = [(IMAGE_COLOR, 16), (IMAGE_NORMAL_MAP, 32), (IMAGE_METALLIC_ROUGHNESS, 8)]
    if texture_workers > 0:
        from concurrent.futures import ThreadPoolExecutor

        base = int(rng.integers(0, 2 ** 63))

        def one(i):
            kind, cells = kinds[i % 3]
            trng = np.random.Generator(np.random.PCG64([base, i]))
            return make_texture(trng, texture_size, kind, cells=cells, separable=True)

        with ThreadPoolExecutor(texture_workers) as ex:
            textures = list(ex.map(one, range(3 * materials)))
    else:
        for k in range(materials):
            for kind, cells in kinds:
                textures.append(make_texture(rng, texture_size, kind, cells=cells))
    for k in range(materials):
        t0 = 3 * k
        mats.append(material(color_image=t0, normal_image=t0 + 1, metallic_image=t0 + 2, sampler=0))
    surf = np.zeros(meshes, SURFACE_DTYPE)
    surf["mesh_index"] = np.arange(meshes)
    surf["graphics_object_index"] = np.arange(meshes)
    surf["material_index"] = rng.integers(0, materials, meshes)
    surf["index_count"] = len(sidx)
    sun_dir = _unit(rng, 1)[0]
    sun_dir[1] = abs(sun_dir[1]) + 0.5
    sun_position, spn = sun_matrices(sun_dir)
    proj = projection(width / height, math.radians(fov_deg))
    cams = []
    for cp in cam_positions:
        target = np.array([rng.uniform(-2, 2), 0.5, rng.uniform(-2, 2)])
        cams.append(scene_record(camera_look_at_origin(cp, target), proj, sun_position, spn, cp,
                                 width, height))
    return Scene(
        name=f"scene_scale_s{seed}_m{meshes}x{triangles_per_mesh}_{width}x{height}",
        width=width, height=height, shadow_size=shadow_size,
        vertices=verts, indices=idx, meshes=mesh_list,
        objects=np.stack(objects), surfaces=surf,
        materials=np.concatenate(mats), textures=textures, samplers=linear_sampler(),
        scene=cams[0], draw_config=default_draw_config(pcf_mode), cameras=cams)


def stress(seed: int = 0, width: int = 3840, height: int = 2160, frames: int = 8, texture_size: int = 2048,
           texture_workers: int = 16) -> Scene:
    """The combined stress workload: 1,048,576 triangles over 256 meshes, 64
    materials with three texture_size^2 textures each (full mips), 4 nested
    shadow cascades of 4096^2 (the light's near extent 9 units, then 18, 36, 72),
    3x3 PCF, `frames` spline cameras (one view each)."""
    s = scene_scale(seed=seed, meshes=256, triangles_per_mesh=4096, materials=64, texture_size=texture_size,
                    width=width, height=height, shadow_size=4096, frames=frames, pcf_mode=PCF_3X3,
                    texture_workers=texture_workers)
    s.name = f"stress_s{seed}_{width}x{height}"
    cams = []
    for c in s.cameras:
        c = c.copy()
        P = c["shadow_projection_near"][0].reshape(4, 4).copy()
        P[:, 0:2] *= 4.0  # near cascade: 36 / 4 = 9 units
        c["shadow_projection_near"] = P.reshape(1, 16)
        cams.append(c)
    s.cameras = cams
    s.scene = cams[0]
    s.draw_config = s.draw_config.copy()
    s.draw_config["shadow_cascades"] = 4
    return s


def tiny(seed: int = 0) -> Scene:
    """A few hundred triangles at 96x64 for fast tests."""
    return random_triangles(seed=seed, triangles=256, width=96, height=64, shadow_size=128,
                            texture_size=64)


def with_blended(s: Scene, fraction: float = 0.5, alpha: float = 0.6, mask_cutoff: float | None = None,
                 seed: int = 0) -> Scene:
    """The same scene with the trailing `fraction` of every surface's triangles
    split off into a blended surface (alpha_mode 2, base colour alpha `alpha`),
    or, with `mask_cutoff`, an alpha-mask surface (alpha_mode 1) whose colour
    texture alpha varies so that some fragments are discarded."""
    rng = np.random.Generator(np.random.PCG64(seed))
    mats = [m for m in s.materials]
    textures = list(s.textures)
    new_mats = []
    for m in s.materials:
        b = m.copy()
        b["alpha_mode"] = 1 if mask_cutoff is not None else 2
        b["alpha_cutoff"] = mask_cutoff if mask_cutoff is not None else 0.0
        b["base_color_factor"][3] = alpha
        if mask_cutoff is not None and b["color_image_index"] != U32_MAX:
            t = textures[int(b["color_image_index"])]
            tex = t.texels.copy().reshape(-1, 4)
            tex[:, 3] = rng.integers(0, 256, len(tex))
            textures.append(Texture(t.width, t.height, t.levels, t.image_type, tex.reshape(-1)))
            b["color_image_index"] = len(textures) - 1
        new_mats.append(b)
    materials = np.concatenate([np.asarray(mats, MATERIAL_DTYPE).reshape(-1), np.asarray(new_mats, MATERIAL_DTYPE).reshape(-1)])
    nm = len(s.materials)
    surfs = []
    for sf in s.surfaces:
        tris = int(sf["index_count"]) // 3
        keep = tris - int(tris * fraction)
        a = sf.copy()
        a["index_count"] = keep * 3
        surfs.append(a)
        if keep < tris:
            b = sf.copy()
            b["start_index"] = sf["start_index"] + keep * 3
            b["index_count"] = (tris - keep) * 3
            b["blended"] = 1
            if sf["material_index"] != U32_MAX:
                b["material_index"] = sf["material_index"] + nm
            surfs.append(b)
    out = Scene(**{k: getattr(s, k) for k in s.__dataclass_fields__})
    out.surfaces = np.asarray(surfs, SURFACE_DTYPE).reshape(-1)
    out.materials = materials
    out.textures = textures
    out.name = s.name + ("_mask" if mask_cutoff is not None else "_blended")
    return out


def view_of(s: Scene, width: int, height: int, shadow_size: int, camera: int = 0, fov_deg: float = 60.0) -> Scene:
    """The scene seen through camera `camera` at another extent and shadow-map size."""
    out = Scene(**{k: getattr(s, k) for k in s.__dataclass_fields__})
    src = s.cameras[camera % len(s.cameras)]
    view = src["view"][0].reshape(4, 4).T.astype(np.float64)
    cam = np.linalg.inv(view)[:3, 3]
    sun = src["sun_position"][0]
    spn = src["shadow_projection_near"][0].reshape(4, 4).T.astype(np.float64)
    proj = projection(width / height, math.radians(fov_deg))
    rec = scene_record(view, proj, sun, spn, cam, width, height)
    for k in ("fragment_output", "light_enabled", "tangent_space_enabled", "shadows_enabled", "normal_maps_enabled",
              "brdf_lighting_enabled", "flip_lights", "flip_tangents"):
        rec[k] = src[k]
    out.scene = rec
    out.cameras = [rec]
    out.width, out.height, out.shadow_size = width, height, shadow_size
    return out


def orbit_view(s: Scene, cam_dir, width: int, height: int, fov_deg: float = 60.0) -> np.ndarray:
    """Scene constants of a camera at 3 * cam_dir looking at the origin (the
    random-triangles camera), keeping the scene's sun and feature switches."""
    src = s.scene
    cam = 3.0 * np.asarray(cam_dir, np.float64) / np.linalg.norm(cam_dir)
    view = camera_look_at_origin(cam)
    spn = src["shadow_projection_near"][0].reshape(4, 4).T.astype(np.float64)
    rec = scene_record(view, projection(width / height, math.radians(fov_deg)), src["sun_position"][0], spn, cam,
                       width, height)
    for k in ("fragment_output", "light_enabled", "tangent_space_enabled", "shadows_enabled", "normal_maps_enabled",
              "brdf_lighting_enabled", "flip_lights", "flip_tangents"):
        rec[k] = src[k]
    return rec


def camera_dirs(count: int, seed: int) -> np.ndarray:
    """`count` seeded unit vectors (camera directions on the orbit sphere)."""
    return _unit(np.random.Generator(np.random.PCG64(seed)), count)


def batch_views(seed: int = 0, views: int = 256, scenes: int = 16, min_tris: int = 1000, max_tris: int = 200000,
                min_size: int = 64, max_size: int = 1024, min_shadow: int = 512, max_shadow: int = 2048,
                texture_size: int = 256):
    """Many views of uneven size over several scenes: `scenes` seeded scenes with
    log-uniform triangle counts in [min_tris, max_tris], and `views` views with
    log-uniform extents in [min_size, max_size]^2 and log-uniform shadow maps in
    [min_shadow, max_shadow]^2, each on a random scene and spline camera.
    Returns (scene list, [(scene index, view Scene)])."""
    rng = np.random.Generator(np.random.PCG64(seed))
    scene_list = []
    for k in range(scenes):
        tris = int(round(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))))
        meshes = int(max(1, min(64, tris // 2048)))
        per = max(128, (tris // meshes) // 128 * 128)
        scene_list.append(scene_scale(seed=seed * 1000 + k, meshes=meshes, triangles_per_mesh=per,
                                      materials=max(1, min(8, meshes)), texture_size=texture_size, width=512,
                                      height=512, shadow_size=min_shadow, frames=8))
    out = []
    for v in range(views):
        k = int(rng.integers(0, scenes))
        w = int(round(math.exp(rng.uniform(math.log(min_size), math.log(max_size)))))
        h = int(round(math.exp(rng.uniform(math.log(min_size), math.log(max_size)))))
        sz = int(round(math.exp(rng.uniform(math.log(min_shadow), math.log(max_shadow)))))
        out.append((k, view_of(scene_list[k], w, h, sz, camera=int(rng.integers(0, 8)))))
    return scene_list, out
