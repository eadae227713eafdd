"""GPU parity at the configurations' full sizes and on the fragment program's
less common branches, against the oracle.

* Material and sampler branches (src/shaders/basic.slang:138-344,
  src/Engine/Graphics.cpp:250-278, 3421-3438): mixmap, draws without a
  material, every filter and wrap code, the default sampler, odd texture sizes.
* Batched views at their stated size: 256 views of 64^2..1024^2 over 16 scenes
  of 1k-200k triangles, each with its own 512^2..2048^2 shadow map, in one
  render call; a seeded sample of views (with the largest view and a view of the
  largest scene) against the oracle rendering each view alone.
* The stress view: 1,048,576 triangles, 64 materials of three 2048^2 textures,
  four 4096^2 shadow cascades, 3840x2160.

Bar as everywhere: triangle ids, depth and shadow maps bit-exact, colour within
1/255 per channel.
"""
import numpy as np
import pytest

from kat_scenes import material_zoo
from rosy_gb300 import scene as sc
from rosy_gb300.graphics import Graphics, render_scene
from test_gpu_parity import COLOR_TOL, check_parity

pytestmark = pytest.mark.gpu


def _check_msaa(ref, out):
    assert np.array_equal(out["ids"], ref["ids"]), f"ids differ at {np.count_nonzero(out['ids'] != ref['ids'])} samples"
    assert np.array_equal(out["vis_depth"].view(np.uint32), ref["depth"].view(np.uint32)), "sample depth differs"
    assert np.array_equal(out["shadow"].view(np.uint32), ref["shadow"].view(np.uint32))
    d = np.abs(out["color"].astype(np.int32) - ref["color"].astype(np.int32))
    assert d.max() <= COLOR_TOL, f"colour differs by {d.max()} at {np.count_nonzero(d > COLOR_TOL)} channels"


ZOO = {
    "zoo_s0": lambda: material_zoo(0),
    "zoo_s1_lambert_3x3": lambda: _lambert_3x3(material_zoo(1, width=256, height=160)),
    "zoo_s2_world_space": lambda: _world_space(material_zoo(2, width=200, height=200)),
    "zoo_s3_blended": lambda: sc.with_blended(material_zoo(3, triangles=1600, width=240, height=150), 0.4,
                                              alpha=0.55),
    "zoo_s4_alpha_mask": lambda: sc.with_blended(material_zoo(4, triangles=1600, width=240, height=150), 0.5,
                                                 alpha=1.0, mask_cutoff=0.45),
}


def _lambert_3x3(s):
    s.scene["brdf_lighting_enabled"] = 0
    s.draw_config["pcf_mode"] = sc.PCF_3X3
    return s


def _world_space(s):
    s.scene["tangent_space_enabled"] = 0
    s.scene["ensure_orthogonal_bitangent"] = 1
    s.scene["ignore_asset_tangent_sign"] = 1
    return s


@pytest.mark.parametrize("name", list(ZOO))
def test_material_and_sampler_branches(gpu, oracle, name):
    s = ZOO[name]()
    ref = oracle.render(s)
    out = render_scene(s)
    # every opaque draw, the material-less one included, shows up in the frame
    # (blended draws leave no triangle ids)
    ids = ref["ids"][ref["ids"] > 0] - 1
    counts = s.surfaces[s.surfaces["blended"] == 0]["index_count"] // 3  # ids run over the opaque list
    ends = np.cumsum(counts)
    for a, b in zip(ends - counts, ends):
        assert ((ids >= a) & (ids < b)).any()
    check_parity(s, ref, out)


@pytest.mark.parametrize("mode", [0, 2, 3, 5, 7, 9, 12])
def test_material_branches_in_debug_outputs(gpu, oracle, mode):
    """The fragment program's debug outputs show the sampled material values
    (albedo, normals, metallic / roughness) directly, without lighting."""
    s = material_zoo(5, triangles=1500, width=160, height=100)
    s.scene["fragment_output"] = mode
    check_parity(s, oracle.render(s), render_scene(s))


def test_material_branches_msaa(gpu, oracle):
    s = sc.with_blended(material_zoo(6, triangles=1200, width=160, height=112), 0.3, alpha=0.5)
    s.samples = 4
    _check_msaa(oracle.render(s), render_scene(s))


def _views_to_check(scenes, views, count=16, seed=11):
    rng = np.random.Generator(np.random.PCG64(seed))
    pick = set(rng.choice(len(views), count, replace=False).tolist())
    pick.add(max(range(len(views)), key=lambda i: views[i][1].width * views[i][1].height))
    pick.add(max(range(len(views)), key=lambda i: views[i][1].shadow_size))
    biggest_scene = max(range(len(scenes)), key=lambda k: scenes[k].triangle_count)
    pick.add(next(i for i, (k, _) in enumerate(views) if k == biggest_scene))
    return sorted(pick)


def test_batched_views_full_size(gpu, oracle):
    """256 views over 16 scenes in one render (one launch per stage over all
    views, one graph); 19 of them against the oracle."""
    scenes, views = sc.batch_views()
    assert len(views) == 256 and len(scenes) == 16
    assert max(s.triangle_count for s in scenes) > 100_000
    g = Graphics()
    g.init(64, 64, 64)
    try:
        idx = [g.add_scene(s) for s in scenes]
        g.set_views([(idx[k], v.width, v.height, v.shadow_size, v.draw_config) for k, v in views])
        for i, (_, v) in enumerate(views):
            g.update_view(i, v.scene)
        g.render()
        if g.sync_code() == 14:  # queues sized from the device's counts, then the frame again
            g.render()
        g.sync()
        for i in _views_to_check(scenes, views):
            v = views[i][1]
            out = g.download_view(i)
            ref = oracle.render(v)
            assert (ref["ids"] > 0).any()
            check_parity(v, ref, out)
    finally:
        g.deinit()


def test_stress_view_full_size(gpu, oracle):
    """One view of the stress workload: 1,048,576 triangles over 256 meshes, 64
    materials with three 2048^2 textures each, 4 nested 4096^2 shadow cascades,
    3x3 PCF, 3840x2160."""
    s = sc.stress(frames=2)
    assert s.triangle_count == 1 << 20 and len(s.textures) == 192
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size)
    try:
        g.set_asset(s)
        g.set_graphic_objects(s.objects, s.surfaces)
        g.set_draw_config(s.draw_config)
        for cam in (0, 1):
            si = s.with_camera(cam)
            g.update(si.scene)
            g.render()
            if g.sync_code() == 14:
                g.render()
            g.sync()
            out = g.download()
            ref = oracle.render(si)
            assert ref["shadow"].shape == (4, 4096, 4096)
            assert (ref["ids"] > 0).mean() > 0.05
            check_parity(si, ref, out)
    finally:
        g.deinit()
