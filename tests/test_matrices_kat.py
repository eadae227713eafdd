"""Known answers of the host-side camera and light matrices (the restatement of
src/Engine/Camera.cpp:62-98 and src/Engine/Level.cpp:455-527 in rosy_gb300/scene.py),
derived by hand from their definitions: reverse-Z depth with Vulkan's y and z flip,
a view that looks at its target, the sun's orthographic shadow projection, and the
object records of src/Engine/Node.cpp."""
import math

import numpy as np
import pytest

from rosy_gb300 import scene as sc


def _ndc(m, p):
    c = m @ np.array([p[0], p[1], p[2], 1.0])
    return c[:3] / c[3], c[3]


@pytest.mark.parametrize("aspect", [16.0 / 9.0, 1.0, 0.5])
def test_projection_reverse_z_and_vulkan_flip(aspect):
    fov = math.radians(60.0)
    P = sc.projection(aspect, fov)
    n, f = sc.NEAR, sc.FAR
    t = math.tan(fov * 0.5)
    # the near plane maps to depth 1 and the far plane to depth 0 (reverse Z)
    (x, y, z), w = _ndc(P, (0.0, 0.0, -n))
    assert abs(z - 1.0) < 1e-12 and abs(w - n) < 1e-12 and x == 0.0 and y == 0.0
    (_, _, z), w = _ndc(P, (0.0, 0.0, -f))
    assert abs(z) < 1e-12 and abs(w - f) < 1e-9
    # depth decreases with distance: nearer fragments win a GREATER_OR_EQUAL test
    zs = [_ndc(P, (0.0, 0.0, -d))[0][2] for d in (0.5, 1.0, 3.0, 10.0, 100.0)]
    assert all(a > b for a, b in zip(zs, zs[1:]))
    for d in (1.0, 7.0):
        # the top edge of the field of view is Vulkan's y = -1 (y points down), the bottom +1
        assert abs(_ndc(P, (0.0, t * d, -d))[0][1] + 1.0) < 1e-12
        assert abs(_ndc(P, (0.0, -t * d, -d))[0][1] - 1.0) < 1e-12
        # the right edge is x = +1, the horizontal extent widened by the aspect ratio
        assert abs(_ndc(P, (aspect * t * d, 0.0, -d))[0][0] - 1.0) < 1e-12


@pytest.mark.parametrize("pos", [(0.0, 0.0, 3.0), (3.0, 0.0, 0.0), (1.0, 2.0, -2.0), (-0.5, -1.2, 2.6)])
def test_view_looks_at_its_target(pos):
    V = sc.camera_look_at_origin(pos)
    d = float(np.linalg.norm(pos))
    # the target is straight ahead (camera space looks down -z), the eye is the origin
    assert np.allclose(V @ np.array([0.0, 0.0, 0.0, 1.0]), [0.0, 0.0, -d, 1.0], atol=1e-12)
    assert np.allclose(V @ np.array([*pos, 1.0]), [0.0, 0.0, 0.0, 1.0], atol=1e-12)
    R = V[:3, :3]
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and abs(np.linalg.det(R) - 1.0) < 1e-12
    # yaw and pitch only: the camera's right axis stays horizontal (no roll)
    right = np.linalg.inv(V)[:3, 0]
    assert abs(right[1]) < 1e-12


@pytest.mark.parametrize("u", [(0.3, 0.8, 0.2), (-0.5, 0.7, -0.5), (0.0, 1.0, 0.0001), (0.9, 0.1, -0.4)])
def test_sun_shadow_projection(u):
    u = np.asarray(u, np.float64) / np.linalg.norm(u)
    sun, S = sc.sun_matrices(u)
    D, depth, level = sc.SUN_DISTANCE, sc.ORTHOGRAPHIC_DEPTH, sc.CASCADE_LEVEL
    # the sun sits sun_distance along the direction, and looks at the origin
    assert np.allclose(sun[:3], D * u, atol=1e-9)
    (x, y, z), w = _ndc(S, (0.0, 0.0, 0.0))
    assert abs(x) < 1e-12 and abs(y) < 1e-12 and abs(z - D / depth) < 1e-12 and w == 1.0
    # orthographic: w stays 1, and a step towards the sun raises the depth linearly,
    # so the surface nearest the light wins the shadow pass's GREATER_OR_EQUAL test
    for t in (-5.0, 2.0, 10.0):
        (_, _, zt), wt = _ndc(S, t * u)
        assert wt == pytest.approx(1.0, abs=1e-12)
        assert zt == pytest.approx((D + t) / depth, abs=1e-12)
    # across the light direction the map spans cascade_level: a point half of it
    # away from the axis lands on the unit circle of (x, y), and keeps the origin's depth
    a = np.cross(u, [0.0, 0.0, 1.0] if abs(u[2]) < 0.9 else [1.0, 0.0, 0.0])
    a /= np.linalg.norm(a)
    b = np.cross(u, a)
    for v in (a, b, (a + b) / math.sqrt(2.0)):
        (x, y, z), _ = _ndc(S, 0.5 * level * v)
        assert math.hypot(x, y) == pytest.approx(1.0, abs=1e-12)
        assert z == pytest.approx(D / depth, abs=1e-12)


def test_node_world_and_object_record():
    t, s, yaw = np.array([1.5, -2.0, 0.25]), 2.5, math.radians(30.0)
    W = sc.node_world(t, s, yaw)
    assert np.allclose(W @ [0.0, 0.0, 0.0, 1.0], [*t, 1.0])
    # T * R(yaw about -y) * S: the object's +x axis turns towards +z
    assert np.allclose(W @ [1.0, 0.0, 0.0, 1.0], [*(t + s * np.array([math.cos(yaw), 0.0, math.sin(yaw)])), 1.0])
    assert np.allclose(W @ [0.0, 1.0, 0.0, 1.0], [*(t + [0.0, s, 0.0]), 1.0])
    rec = sc.object_record(W)
    world = rec[0:16].reshape(4, 4).T.astype(np.float64)  # column-major, as glm stores it
    to_object = rec[16:32].reshape(4, 4).T.astype(np.float64)
    normal = rec[32:41].reshape(3, 3).T.astype(np.float64)
    assert np.allclose(world, W, atol=1e-6)
    assert np.allclose(world @ to_object, np.eye(4), atol=1e-5)
    # the normal matrix is the inverse transpose of the upper 3x3: rotation / scale here
    assert np.allclose(normal, np.linalg.inv(W[:3, :3]).T, atol=1e-6)
    n = normal @ np.array([1.0, 0.0, 0.0])
    assert np.allclose(n, np.array([math.cos(yaw), 0.0, math.sin(yaw)]) / s, atol=1e-6)
