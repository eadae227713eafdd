"""GPU tests of the learned upsampler's tensor-core kernels against the numpy
oracle (oracle/upsampler_ref.py): the tcgen05 GEMM layout, the G-buffer the
shading pass writes, the forward pass, the gradients of every parameter, the
Adam step, and that a few training steps lower the loss."""
import numpy as np
import pytest

from oracle import upsampler_ref as U
from rosy_gb300 import scene as sc
from rosy_gb300 import upsampler as up
from rosy_gb300.graphics import Graphics

pytestmark = pytest.mark.gpu


def _render(s, gbuffer=True):
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size)
    g.set_asset(s)
    g.set_graphic_objects(s.objects, s.surfaces)
    g.set_draw_config(s.draw_config)
    if gbuffer:
        g.set_gbuffer(True)
    g.update(s.scene)
    g.render()
    if g.sync_code() == 14:
        g.render()
    g.sync()
    return g


def _pair(w, h, camera=0, seed=0):
    """Half-resolution G-buffer renderer and the full-resolution target of one camera."""
    base = sc.tiny(seed)
    lo = _render(sc.view_of(base, w, h, 128, camera=camera))
    hi = _render(sc.view_of(base, 2 * w, 2 * h, 128, camera=camera), gbuffer=False)
    return lo, hi


def _params(seed, last_scale=0.2):
    rng = np.random.default_rng(seed)
    p = U.init_params(seed, last_scale=last_scale)
    for (wo, bo), (cin, cout) in zip(U.OFFSETS, U.LAYERS):
        real = 12 if cout == 16 else cout
        p[bo:bo + real] = rng.normal(0.0, 0.05, real).astype(np.float32)
    return p


def test_tcgen05_selftest_gemm(gpu):
    import torch

    for n in (16, 32):
        for k in (16, 64):
            gen = torch.Generator().manual_seed(100 * n + k)
            A = torch.randn(128, k, generator=gen).to(torch.bfloat16)
            B = torch.randn(n, k, generator=gen).to(torch.bfloat16)
            a, b = A.cuda(), B.cuda()
            d = torch.full((128, n), float("nan"), device="cuda")
            torch.cuda.synchronize()
            assert up.selftest_gemm(a.data_ptr(), b.data_ptr(), d.data_ptr(), n, k) == 0
            want = A.double() @ B.double().T
            err = (d.cpu().double() - want).abs().max().item()
            assert err < 1e-3 * max(1.0, want.abs().max().item()), (n, k, err)


def test_gbuffer_albedo_and_normal(gpu):
    s = sc.tiny(0)
    s.scene = s.scene.copy()
    s.scene["light_enabled"] = 0
    s.scene["fragment_output"] = 0
    g = _render(s)
    gb = g.download_gbuffer()
    fr = g.download()
    covered = fr["ids"] > 0
    assert covered.any() and (~covered).any()
    assert np.array_equal(gb["albedo"][..., 3], np.where(covered, 255, 0).astype(np.uint8))
    # unlit, debug output 0: the colour is the sampled albedo
    assert np.array_equal(gb["albedo"][covered][:, :3], fr["color"][covered][:, :3])
    assert np.array_equal(gb["color"], fr["color"])
    # debug output 1 shows the world normal * 0.5 + 0.5; compare with the decoded octahedral normal
    s.scene["fragment_output"] = 1
    g.update(s.scene)
    g.render()
    g.sync()
    col = g.download()["color"][..., :3].astype(np.float64) / 255.0
    lin = np.where(col <= 0.04045, col / 12.92, ((col + 0.055) / 1.055) ** 2.4)
    n_dbg = lin[covered] * 2.0 - 1.0
    o = gb["normal"][covered].astype(np.float64)
    z = 1.0 - np.abs(o[:, 0]) - np.abs(o[:, 1])
    x, y = o[:, 0].copy(), o[:, 1].copy()
    neg = z < 0
    x[neg] = (1.0 - np.abs(o[neg, 1])) * np.sign(o[neg, 0])
    y[neg] = (1.0 - np.abs(o[neg, 0])) * np.sign(o[neg, 1])
    n = np.stack([x, y, z], 1)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    err = np.abs(n - n_dbg)
    assert err.mean() < 0.01 and err.max() < 0.06, (err.mean(), err.max())
    g.deinit()


def _orbit(s, cam, w, h):
    out = sc.Scene(**{k: getattr(s, k) for k in s.__dataclass_fields__})
    out.width, out.height = w, h
    out.scene = sc.orbit_view(s, sc.camera_dirs(8, 2002)[cam], w, h)
    out.cameras = [out.scene]
    return out


def _inside():  # the camera inside the cube: triangles cut by the near plane
    s = sc.random_triangles(seed=3, triangles=2000, width=320, height=200, shadow_size=256, texture_size=32)
    view = sc.camera_look_at_origin((0.2, 0.1, 0.3))
    proj = sc.projection(320 / 200, np.radians(90.0))
    s.scene = sc.scene_record(view, proj, s.scene["sun_position"][0], np.eye(4), (0.2, 0.1, 0.3), 320, 200)
    s.scene["shadow_projection_near"] = s.cameras[0]["shadow_projection_near"]
    s.cameras = [s.scene]
    return s


SUBPIXEL = {
    "random_triangles_960x540": lambda: _orbit(sc.random_triangles(seed=0, width=1920, height=1080), 3, 960, 540),
    "scene_scale_small": lambda: sc.scene_scale(seed=6, meshes=8, triangles_per_mesh=512, materials=3,
                                                texture_size=32, width=320, height=180, shadow_size=256, frames=1),
    "camera_inside_clipping": _inside,
}


@pytest.mark.parametrize("name", list(SUBPIXEL))
def test_subpixel_sources_match_oracle(gpu, oracle, name):
    """The G-buffer's sub-pixel sources (k_subpixel_sources) equal the oracle's
    restatement bit for bit, from the same visibility."""
    s = SUBPIXEL[name]()
    g = _render(s)
    try:
        fr = g.download()
        gb = g.download_gbuffer()
        ref_ids = oracle.raster(s)["ids"]
        assert np.array_equal(fr["ids"], ref_ids)
        want = oracle.subpixel_sources(s, ref_ids)
        assert (want != 0xFFFF).mean() > 0.01
        assert np.array_equal(gb["sources"], want), f"{np.count_nonzero(gb['sources'] != want)} masks differ"
    finally:
        g.deinit()


def test_subpixel_sources_in_batched_views_and_not_with_msaa(gpu, oracle):
    """Per view of a batch (triangle ids are global; each view's plane resolves
    them through the whole draw list) the sources equal the oracle's for that view
    alone; multisampled frames have no sources plane (plain bilinear base)."""
    scenes, views = sc.batch_views(seed=8, views=4, scenes=2, min_tris=800, max_tris=5000, min_size=60,
                                   max_size=240, min_shadow=128, max_shadow=256, texture_size=32)
    g = Graphics()
    g.init(64, 64, 64)
    try:
        idx = [g.add_scene(x) for x in scenes]
        g.set_views([(idx[k], v.width, v.height, v.shadow_size, v.draw_config) for k, v in views])
        g.set_gbuffer(True)
        for i, (_, v) in enumerate(views):
            g.update_view(i, v.scene)
        g.render()
        if g.sync_code() == 14:
            g.render()
        g.sync()
        for i, (_, v) in enumerate(views):
            local = g.download_view(i)["ids"]  # triangle ids of the view alone
            want = oracle.subpixel_sources(v, local)
            assert (want != 0xFFFF).any()
            assert np.array_equal(g.download_gbuffer(i)["sources"], want)
    finally:
        g.deinit()
    s = sc.tiny(2)
    s.samples = 4
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size, samples=4)
    try:
        g.set_asset(s)
        g.set_graphic_objects(s.objects, s.surfaces)
        g.set_draw_config(s.draw_config)
        g.set_gbuffer(True)
        g.update(s.scene)
        g.render()
        g.sync()
        assert "sources" not in g.download_gbuffer()
    finally:
        g.deinit()


@pytest.mark.parametrize("w,h", [(96, 64), (200, 70), (960, 540)])
def test_upsampler_forward_matches_oracle(gpu, w, h):
    import torch

    lo, hi = _pair(w, h)
    gbh = lo.download_gbuffer()
    p = _params(5)
    u = up.Upsampler(0, w, h)
    u.set_params(p)
    out = torch.zeros((2 * h, 2 * w), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    u.infer(lo.gbuffer(), out.data_ptr())
    assert u.status() == 0
    got = out.cpu().numpy().view(np.uint8).reshape(2 * h, 2 * w, 4)
    ref = U.forward(p, gbh)["rgba8"]
    d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
    assert d.max() <= 2 and (d > 0).mean() < 0.01, (d.max(), (d > 0).mean())
    # the prediction differs from plain bilinear (the network did something)
    assert not np.array_equal(ref, U.to_rgba8(U.bilinear_base(gbh["color"])))
    u.close()
    lo.deinit()
    hi.deinit()


def test_zero_network_is_exactly_the_x2_base(gpu):
    """With every parameter zero the network adds nothing, so the output is the
    x2 base alone, and it equals the oracle's bit for bit: byte / 255, the
    9/16, 3/16, 3/16, 1/16 sum in order over the sub-pixel sources that show
    each point's triangle, renormalised, clamping and rounding to 8 bits; and
    plain bilinear when the G-buffer has no sources."""
    import torch

    w, h = 200, 70
    lo, hi = _pair(w, h, camera=3)
    gbh = lo.download_gbuffer()
    u = up.Upsampler(0, w, h)
    u.set_params(np.zeros_like(U.init_params(0)))
    out = torch.zeros((2 * h, 2 * w), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    u.infer(lo.gbuffer(), out.data_ptr())
    assert u.status() == 0
    got = out.cpu().numpy().view(np.uint8).reshape(2 * h, 2 * w, 4)
    assert "sources" in gbh and (gbh["sources"] != 0xFFFF).any()
    assert np.array_equal(got, U.to_rgba8(U.x2_base(gbh["color"], gbh["sources"])))
    assert not np.array_equal(got, U.to_rgba8(U.bilinear_base(gbh["color"])))
    g = lo.gbuffer()
    g.sources_u16 = None
    u.infer(g, out.data_ptr())
    assert u.status() == 0
    got = out.cpu().numpy().view(np.uint8).reshape(2 * h, 2 * w, 4)
    assert np.array_equal(got, U.to_rgba8(U.bilinear_base(gbh["color"])))
    u.close()
    lo.deinit()
    hi.deinit()


@pytest.mark.parametrize("w,h", [(96, 64), (200, 70), (960, 540)])
def test_upsampler_gradients_match_oracle(gpu, w, h):
    import torch

    lo, hi = _pair(w, h, camera=1)
    gbh = lo.download_gbuffer()
    target = hi.download()["color"]
    p = _params(9)
    u = up.Upsampler(0, w, h)
    u.set_params(p)
    tgt = torch.from_numpy(target.reshape(2 * h, 2 * w, 4).view(np.int32).reshape(2 * h, 2 * w).copy()).cuda()
    torch.cuda.synchronize()
    u.accumulate(lo.gbuffer(), tgt.data_ptr())
    grads, loss, values = u.grads()
    assert u.status() == 0
    assert values == 2 * h * 2 * w * 3
    ref, ref_loss = U.gradients(p, gbh, target)
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss, (loss, ref_loss)
    for l, ((wo, bo), (cin, cout)) in enumerate(zip(U.OFFSETS, U.LAYERS)):
        for name, sl in (("w", slice(wo, bo)), ("b", slice(bo, bo + cout))):
            a, r = grads[sl].astype(np.float64), ref[sl]
            rel = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-12)
            assert rel < 2e-2, (l, name, rel)
    # Adam, first step: p - lr * g / (|g| + eps) with bias-corrected moments
    lr = 1e-3
    u.adam_step(lr, 0.9, 0.999, 1e-8, 1.0)
    p1 = u.params()
    g64 = grads.astype(np.float64)
    want = p - lr * g64 / (np.abs(g64) + 1e-8)
    assert np.allclose(p1, want, rtol=1e-5, atol=1e-6)
    _, l2, v2 = u.grads()
    assert l2 == 0.0 and v2 == 0
    u.close()
    lo.deinit()
    hi.deinit()


def test_training_steps_lower_the_loss(gpu):
    import torch

    w, h = 96, 64
    lo, hi = _pair(w, h, camera=2)
    target = hi.download()["color"]
    u = up.Upsampler(0, w, h)
    u.set_params(up.init_params(0))
    tgt = torch.from_numpy(target.view(np.int32).reshape(2 * h, 2 * w).copy()).cuda()
    torch.cuda.synchronize()
    losses = []
    for _ in range(40):
        u.accumulate(lo.gbuffer(), tgt.data_ptr())
        loss, values = u.loss()
        losses.append(loss / values)
        u.adam_step(2e-3, grad_scale=1.0 / values)
    assert u.status() == 0
    assert losses[-1] < 0.8 * losses[0], losses
    u.close()
    lo.deinit()
    hi.deinit()


@pytest.mark.parametrize("samples", [1, 4])
def test_trained_network_beats_bilinear_on_heldout_cameras(gpu, samples):
    """The committed weights (trained only on plain-path frames from the training
    cameras) against the method without the network (bilinear x2, the network with a
    zero last layer), judged by the plain full-resolution render on held-out cameras;
    with the reference's 4x multisampling the network also clears the 38 dB floor."""
    from rosy_gb300 import learned

    params, meta = learned.load_weights(learned.WEIGHTS if samples == 1 else learned.WEIGHTS_MSAA4)
    ev = learned.evaluate(params, cameras=16, samples=samples)
    assert ev["frames"] == 16
    gains = [f["psnr_db"] - f["bilinear_psnr_db"] for f in ev["per_frame"]]
    assert min(gains) > 0.0, gains
    assert ev["psnr_db_mean"] > ev["bilinear_psnr_db_mean"] + 1.0, ev
    if samples == 4:
        assert ev["psnr_db_mean"] >= learned.PSNR_FLOOR_DB, ev
