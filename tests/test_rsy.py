"""The .rsy reader (rz_rsy_* in the C ABI) against files written in the layout of
rosy_asset::asset::write: records, the flattened root scene (static objects,
then mobs) with its transforms, error handling, and rendering a loaded asset."""
import math
import os
import struct

import numpy as np
import pytest

from rosy_gb300 import rsy
from rosy_gb300 import scene as sc
from rosy_gb300._lib import RzError


def _trs(t, yaw, s):
    c, sn = math.cos(-yaw), math.sin(-yaw)
    R = np.array([[c, 0, sn, 0], [0, 1, 0, 0], [-sn, 0, c, 0], [0, 0, 0, 1.0]])
    T = np.eye(4)
    T[:3, 3] = t
    return T @ R @ np.diag([s, s, s, 1.0])


def _asset():
    base = sc.tiny(0)
    pos = base.vertices.reshape(-1, 16)
    idx = base.indices
    half = (len(idx) // 3 // 2) * 3
    mats = np.concatenate([base.materials, base.materials])
    mats[1]["alpha_mode"] = 2  # the second surface goes to the blended list
    mats[1]["double_sided"] = 1
    mesh = rsy.RsyMesh(pos, idx, [(0, half, 0, (-1, -1, -1), (1, 1, 1)), (half, len(idx) - half, 1, (-1, -1, -1),
                                                                         (1, 1, 1))])
    m_a = np.array([[1, 0, 0, 0.2], [0, 1, 0, -0.1], [0, 0, 1, 0.3], [0, 0, 0, 1.0]])
    m_b = np.array([[0.9, 0, 0, 0], [0, 0.9, 0, 0.4], [0, 0, 0.9, 0], [0, 0, 0, 1.0]])
    nodes = [
        rsy.RsyNode((0.5, 0.0, -0.2), 1.2, 0.3, m_a, 0, [1], "root_a"),
        rsy.RsyNode((0.0, 0.1, 0.0), 1.0, 0.0, m_b, 0, [], "child_b"),
        rsy.RsyNode((0.0, 0.0, 0.0), 1.0, 0.0, np.eye(4), 0xFFFFFFFF, [4], "world"),
        rsy.RsyNode((-0.3, 0.0, 0.0), 0.8, -0.5, np.eye(4), 0, [], "m1"),
        rsy.RsyNode((0.0, 0.0, 0.0), 1.0, 0.0, np.eye(4), 0xFFFFFFFF, [3], "mobs"),
    ]
    coord = np.diag([1.0, 1.0, -1.0, 1.0])
    return rsy.RsyAsset(materials=mats, samplers=base.samplers, scenes=[[0, 2]], nodes=nodes,
                        images=[(0, "albedo.dds")], meshes=[mesh], coordinate_system=coord), base


def _expected_worlds(a):
    """World transforms in the order the level emits them: statics then mobs."""
    C = a.coordinate_system
    out_static, out_mob = [], []
    queue = [(n, np.eye(4), False) for n in a.scenes[a.root_scene]]
    while queue:
        i, parent, mob = queue.pop(0)
        n = a.nodes[i]
        obj = parent @ n.transform
        world = _trs(n.world_translate, n.world_yaw, n.world_scale) @ C @ obj
        if n.mesh_id != 0xFFFFFFFF:
            (out_mob if mob else out_static).append(world)
        for c in n.children:
            queue.append((c, obj, mob or a.nodes[c].name == "mobs"))
    return out_static, out_mob


def test_rsy_round_trip_and_scene(tmp_path, renderer_lib):
    a, base = _asset()
    p = str(tmp_path / "level.rsy")
    rsy.write_rsy(p, a)
    f = rsy.RsyFile(p)
    info = f.info
    assert (info.mesh_count, info.material_count, info.sampler_count, info.image_count, info.node_count,
            info.scene_count) == (1, 2, 1, 1, 5, 1)
    assert np.allclose(np.array(info.coordinate_system).reshape(4, 4).T, a.coordinate_system)
    (pos, idx), = f.meshes()
    assert np.array_equal(pos, a.meshes[0].positions.astype(np.float32)) and np.array_equal(idx, a.meshes[0].indices)
    assert f.materials().tobytes() == a.materials.tobytes()
    assert f.samplers().tobytes() == a.samplers.tobytes()
    assert f.images() == [(0, "albedo.dds")]
    objs, surfs = f.scene_objects()
    statics, mobs = _expected_worlds(a)
    assert info.static_object_count == len(statics) == 2 and info.object_count == 3
    for k, w in enumerate(statics + mobs):
        got = objs[k, :16].reshape(4, 4).T
        assert np.allclose(got, w, atol=1e-6), k
        assert np.allclose(objs[k, 16:32].reshape(4, 4).T, np.linalg.inv(w), atol=1e-5)
        nrm = np.linalg.inv(w[:3, :3]).T
        assert np.allclose(objs[k, 32:41].reshape(3, 3).T, nrm, atol=1e-5)
    # one surface per mesh surface; mobs index from 0 with the static count as offset
    assert len(surfs) == 6
    assert list(surfs["graphics_object_index"]) == [0, 0, 1, 1, 0, 0]
    assert list(surfs["graphic_objects_offset"]) == [0, 0, 0, 0, 2, 2]
    assert list(surfs["blended"]) == [0, 1, 0, 1, 0, 1]
    assert list(surfs["material_index"]) == [0, 1, 0, 1, 0, 1]
    f.close()


def test_rsy_errors(tmp_path, renderer_lib):
    a, _ = _asset()
    p = str(tmp_path / "ok.rsy")
    rsy.write_rsy(p, a)
    data = open(p, "rb").read()
    with pytest.raises(RzError) as e:
        rsy.RsyFile(str(tmp_path / "missing.rsy"))
    assert e.value.code == 8  # open_failed
    cases = {
        "magic": b"XXXX" + data[4:],
        "version": data[:4] + struct.pack("<I", 2) + data[8:],
        "endianness": data[:8] + struct.pack("<I", 0) + data[12:],
        "truncated": data[:len(data) - 7],
        "header_only": data[:40],
        "huge_count": data[:80] + struct.pack("<Q", 1 << 40) + data[88:],
    }
    for name, blob in cases.items():
        q = str(tmp_path / f"{name}.rsy")
        open(q, "wb").write(blob)
        with pytest.raises(RzError) as e:
            rsy.RsyFile(q)
        assert e.value.code == 11, name  # read_failed
    # a root scene out of range reads, but has no scene
    bad = rsy.RsyAsset(a.materials, a.samplers, a.scenes, a.nodes, a.images, a.meshes, a.coordinate_system, 5)
    q = str(tmp_path / "root.rsy")
    rsy.write_rsy(q, bad)
    f = rsy.RsyFile(q)
    with pytest.raises(RzError) as e:
        f.scene_objects()
    assert e.value.code == 3
    f.close()


def test_rsy_scene_renders_like_the_source_scene(tmp_path, oracle):
    a, base = _asset()
    p = str(tmp_path / "level.rsy")
    rsy.write_rsy(p, a)
    s = rsy.scene_from_rsy(p, textures=base.textures, width=96, height=64, shadow_size=128,
                           camera_position=(0.0, 1.0, 3.5))
    # the same scene assembled by hand from the writer's inputs
    statics, mobs = _expected_worlds(a)
    ref = sc.Scene(**{k: getattr(s, k) for k in s.__dataclass_fields__})
    ref.objects = np.stack([sc.object_record(w) for w in statics + mobs])
    r1 = oracle.raster(s)
    r2 = oracle.raster(ref)
    assert (r1["ids"] > 0).mean() > 0.05
    assert np.array_equal(r1["ids"], r2["ids"]) or np.mean(r1["ids"] != r2["ids"]) < 1e-3


@pytest.mark.gpu
def test_rsy_scene_gpu_matches_oracle(tmp_path, gpu, oracle):
    from rosy_gb300.graphics import render_scene

    a, base = _asset()
    p = str(tmp_path / "level.rsy")
    rsy.write_rsy(p, a)
    s = rsy.scene_from_rsy(p, textures=base.textures, width=96, height=64, shadow_size=128,
                           camera_position=(0.0, 1.0, 3.5))
    got = render_scene(s)
    want = oracle.render(s)
    assert np.array_equal(got["ids"], want["ids"])
    assert np.array_equal(got["depth"], want["depth"])
    assert np.abs(got["color"].astype(int) - want["color"].astype(int)).max() <= 1


def test_rsy_reader_survives_mutated_files(tmp_path, renderer_lib):
    """Random byte edits and truncations of a valid file: the reader returns a
    result code or an asset whose counts are consistent, never crashes."""
    pytest.importorskip("hypothesis")
    from hypothesis import given, settings
    from hypothesis import strategies as st

    a, _ = _asset()
    path = str(tmp_path / "good.rsy")
    rsy.write_rsy(path, a)
    good = open(path, "rb").read()
    bad = str(tmp_path / "bad.rsy")

    @settings(max_examples=200, deadline=None, derandomize=True)
    @given(st.lists(st.tuples(st.integers(0, len(good) - 1), st.integers(0, 255)), max_size=6),
           st.integers(0, len(good)))
    def mutated(edits, cut):
        data = bytearray(good)
        for pos, val in edits:
            data[pos] = val
        with open(bad, "wb") as f:
            f.write(bytes(data[:cut]))
        try:
            f = rsy.RsyFile(bad)
        except RzError as e:
            assert e.code in (3, 11)
            return
        try:
            meshes = f.meshes()
            assert len(meshes) == f.info.mesh_count
            assert len(f.materials()) == f.info.material_count
            f.images()
            try:
                f.scene_objects()
            except RzError as e:  # a damaged scene graph is reported, not followed
                assert e.code == 3
        finally:
            f.close()

    mutated()


GOLDEN_RSY = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rsy")
GOLDEN_CASES = sorted(f[:-4] for f in os.listdir(GOLDEN_RSY) if f.endswith(".rsy"))


class _JsonAsset:
    """The asset the reference's own asset::read decoded, in the shape _expected_worlds wants."""

    def __init__(self, d):
        self.coordinate_system = np.array(d["coordinate_system"], np.float64).reshape(4, 4).T
        self.root_scene = d["root_scene"]
        self.scenes = d["scenes"]
        self.nodes = [rsy.RsyNode(n["world_translate"], n["world_scale"], n["world_yaw"],
                                  np.array(n["transform"], np.float64).reshape(4, 4).T, n["mesh_id"], n["children"],
                                  n["name"]) for n in d["nodes"]]


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_reader_matches_files_the_reference_wrote(renderer_lib, case):
    """Files written by the reference's asset::write (src/Asset/Asset.cpp:28-407,
    compiled from its sources by oracle/ref_rsy, fixtures made by
    tests/golden/make_rsy_golden.py): rz_rsy_read decodes every record to the
    values the reference's own asset::read decoded, and flattens the root scene
    by the level's rules."""
    import json

    d = json.load(open(os.path.join(GOLDEN_RSY, case + ".json")))
    f = rsy.RsyFile(os.path.join(GOLDEN_RSY, case + ".rsy"))
    info = f.info
    assert (info.mesh_count, info.material_count, info.sampler_count, info.image_count, info.node_count,
            info.scene_count, info.root_scene) == (len(d["meshes"]), len(d["materials"]), len(d["samplers"]),
                                                   len(d["images"]), len(d["nodes"]), len(d["scenes"]),
                                                   d["root_scene"])
    assert np.array_equal(np.array(info.coordinate_system, np.float32), np.array(d["coordinate_system"], np.float32))
    for (pos, idx), m in zip(f.meshes(), d["meshes"]):
        assert np.array_equal(pos.reshape(-1), np.array(m["positions"], np.float32))
        assert np.array_equal(idx, np.array(m["indices"], np.uint32))
    mats = f.materials()
    for got, m in zip(mats, d["materials"]):
        assert np.array_equal(got["base_color_factor"], np.array(m["base_color_factor"], np.float32))
        assert got["metallic_factor"] == np.float32(m["metallic_factor"])
        assert got["roughness_factor"] == np.float32(m["roughness_factor"])
        assert got["alpha_cutoff"] == np.float32(m["alpha_cutoff"])
        assert got["alpha_mode"] == m["alpha_mode"] and got["double_sided"] == m["double_sided"]
        names = ("color_image_index", "color_sampler_index", "normal_image_index", "normal_sampler_index",
                 "metallic_image_index", "metallic_sampler_index", "mixmap_image_index", "mixmap_sampler_index")
        assert [int(got[n]) for n in names] == m["indices"]
    smp = f.samplers()
    assert [[int(s[k]) for k in ("min_filter", "mag_filter", "wrap_s", "wrap_t")] for s in smp] == d["samplers"]
    assert f.images() == [(im["type"], im["name"]) for im in d["images"]]
    objs, surfs = f.scene_objects()
    a = _JsonAsset(d)
    statics, mobs = _expected_worlds(a)
    assert info.static_object_count == len(statics) and info.object_count == len(statics) + len(mobs)
    for k, w in enumerate(statics + mobs):
        assert np.allclose(objs[k, :16].reshape(4, 4).T, w, atol=1e-5), k
    # one surface per mesh surface of every object, with the mesh surface's material and range
    want = []
    queue = [(n, False) for n in d["scenes"][d["root_scene"]]]
    order_static, order_mob = [], []
    while queue:
        i, mob = queue.pop(0)
        n = d["nodes"][i]
        if n["mesh_id"] != 0xFFFFFFFF:
            (order_mob if mob else order_static).append(n["mesh_id"])
        queue += [(c, mob or d["nodes"][c]["name"] == "mobs") for c in n["children"]]
    for mesh_id in order_static + order_mob:
        for s in d["meshes"][mesh_id]["surfaces"]:
            want.append((s["material"], s["count"], s["start_index"],
                         int(d["materials"][s["material"]]["alpha_mode"] != 0)))
    assert [(int(s["material_index"]), int(s["index_count"]), int(s["start_index"]), int(s["blended"]))
            for s in surfs] == want
    f.close()
