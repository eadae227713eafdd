"""Bounded waits, made to run out on purpose without faulting or hanging a GPU.

* The blended list's ordered setup waits on its predecessors' look-back words;
  with the bound lowered to one spin some wait gives up, the frame reports
  RZ_GRAPHICS_FRAME_FAILURE with the look-back bit, the blended list is left
  out of that frame, and the next frame with the default bound is exact.
* The upsampler's kernels wait on TMA copies, MMA completions and drained
  accumulators; with a limit of one clock cycle the waits run out, the status
  bit is set, every kernel still returns (after its copies and MMAs in flight
  complete), and a later call with the default limit matches the oracle.
* rz_sync with a timeout returns RZ_TIMEOUT while a frame is still queued
  behind a 0.3 s kernel on the context's stream, and RZ_OK once it is done.
"""
import numpy as np
import pytest

from oracle import upsampler_ref as U
from rosy_gb300 import scene as sc
from rosy_gb300 import upsampler as up
from rosy_gb300.graphics import Graphics
from test_gpu_parity import check_parity

pytestmark = pytest.mark.gpu

RZ_OK, RZ_GRAPHICS_FRAME_FAILURE, RZ_TIMEOUT = 0, 6, 16
ERR_LOOKBACK_TIMEOUT = 1 << 2


def _context(s):
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size)
    g.set_asset(s)
    g.set_graphic_objects(s.objects, s.surfaces)
    g.set_draw_config(s.draw_config)
    g.update(s.scene)
    return g


def test_lookback_wait_runs_out_then_next_frame_is_exact(gpu, oracle):
    # about 100,000 small blended triangles: ~400 ordered setup tiles, many of which
    # find a predecessor that has not published yet
    s = sc.with_blended(sc.scene_scale(seed=61, meshes=64, triangles_per_mesh=2048, materials=4, texture_size=32,
                                       width=256, height=160, shadow_size=512, frames=1), 0.75, alpha=0.5)
    g = _context(s)
    try:
        g.render()
        if g.sync_code() == 14:
            g.render()
        g.sync()
        g.set_wait_limit(1)
        seen = False
        for _ in range(5):
            g.render()
            rc = g.sync_code()
            if rc == RZ_GRAPHICS_FRAME_FAILURE:
                assert g.stats().error_flags & ERR_LOOKBACK_TIMEOUT
                seen = True
                break
            assert rc == RZ_OK
        assert seen, "no look-back wait ran out in 5 frames"
        g.set_wait_limit(0)
        g.render()
        assert g.sync_code() == RZ_OK
        check_parity(s, oracle.render(s), g.download())
    finally:
        g.deinit()


def _gbuffer_frame(w, h):
    s = sc.view_of(sc.tiny(3), w, h, 128, camera=2)
    g = _context(s)
    g.set_gbuffer(True)
    g.render()
    g.sync()
    return g


def test_upsampler_waits_run_out_then_default_limit_is_exact(gpu):
    import torch

    w, h = 200, 70
    g = _gbuffer_frame(w, h)
    try:
        gbh = g.download_gbuffer()
        p = U.init_params(7, last_scale=0.2)
        ref = U.forward(p, gbh)["rgba8"]
        out = torch.zeros((2 * h, 2 * w), dtype=torch.int32, device="cuda")
        tgt = torch.zeros((2 * h, 2 * w), dtype=torch.int32, device="cuda")
        u = up.Upsampler(0, w, h)
        u.set_params(p)
        u.set_wait_limit(1)
        torch.cuda.synchronize()
        u.infer(g.gbuffer(), out.data_ptr())
        u.accumulate(g.gbuffer(), tgt.data_ptr())  # the weight-gradient kernels wait too
        assert u.status() & 1, "no wait ran out with a one-cycle limit"
        # the same object with the default limit again computes the exact output
        # (its status bit stays set), and so does a fresh one
        u.set_wait_limit(0)
        u.infer(g.gbuffer(), out.data_ptr())
        u.status()
        got = out.cpu().numpy().view(np.uint8).reshape(2 * h, 2 * w, 4)
        d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
        assert d.max() <= 2 and (d > 0).mean() < 0.01, (d.max(), (d > 0).mean())
        u.close()
        v = up.Upsampler(0, w, h)
        v.set_params(p)
        out.zero_()
        torch.cuda.synchronize()
        v.infer(g.gbuffer(), out.data_ptr())
        assert v.status() == 0
        got = out.cpu().numpy().view(np.uint8).reshape(2 * h, 2 * w, 4)
        d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
        assert d.max() <= 2 and (d > 0).mean() < 0.01, (d.max(), (d > 0).mean())
        v.close()
    finally:
        g.deinit()


def test_sync_times_out_behind_a_long_kernel(gpu):
    import torch

    s = sc.tiny(4)
    g = _context(s)
    try:
        g.render()
        g.sync()
        stream = torch.cuda.ExternalStream(g.stream)
        with torch.cuda.stream(stream):
            torch.cuda._sleep(int(0.3 * 2.1e9))  # a kernel of about 0.3 s on the context's stream
        g.render()
        assert g.sync_code(10) == RZ_TIMEOUT
        assert g.sync_code(0) == RZ_OK
    finally:
        g.deinit()
