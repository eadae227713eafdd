"""The learned half-resolution path: render a view at W x H with the plain
renderer (G-buffer on), then reconstruct 2W x 2H with the upsampler network.

The network is trained only on frames the plain full-resolution path renders
from seeded cameras on the radius-3 orbit of the random-triangles scene
(4,096 training directions), and judged against the plain full-resolution
render on 256 held-out directions. The plain render stays the reference and
the fallback: `LearnedPath.render` returns the plain full-resolution frame
unless every held-out frame of the network reaches the quality floor.

In single-sample mode the network adds a residual to a triangle-aware x2 base:
the renderer marks, per half-resolution pixel, which bilinear sources show the
triangle in front at each full-resolution pixel centre (the G-buffer's sub-pixel
sources), and the base renormalises the bilinear weights over those.

    python -m rosy_gb300.learned train --steps 3000 --out weights.npz
    python -m rosy_gb300.learned eval --weights weights.npz
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import scene as sc
from .graphics import Graphics
from .upsampler import PARAM_COUNT, Upsampler, conv_flops, init_params

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights", "upsampler_random_triangles.npz")
WEIGHTS_MSAA4 = os.path.join(HERE, "weights", "upsampler_random_triangles_msaa4.npz")
TRAIN_CAMERAS = 4096
TEST_CAMERAS = 256
TRAIN_CAMERA_SEED = 1001
TEST_CAMERA_SEED = 2002
PSNR_FLOOR_DB = 38.0
L2_FLUSH_BYTES = 256 << 20


def _render(g: Graphics, sync: bool) -> None:
    g.render()
    if sync:
        if g.sync_code() == 14:  # the raster queue grew: render again
            g.render()
        g.sync()


class PairRenderer:
    """Two contexts on one scene: `low` at W x H with the G-buffer on, `high` at 2W x 2H,
    both with `samples` camera-pass samples per pixel."""

    def __init__(self, s: sc.Scene, width: int, height: int, device: int = 0, samples: int = 1):
        self.s, self.width, self.height = s, width, height
        self.low = Graphics()
        self.low.init(width, height, s.shadow_size, device, samples=samples)
        self.high = Graphics()
        self.high.init(2 * width, 2 * height, s.shadow_size, device, samples=samples)
        for g in (self.low, self.high):
            g.set_asset(s)
            g.set_graphic_objects(s.objects, s.surfaces)
            g.set_draw_config(s.draw_config)
        self.low.set_gbuffer(True)

    def render_low(self, d, sync: bool = True) -> None:
        self.low.update(sc.orbit_view(self.s, d, self.width, self.height))
        _render(self.low, sync)

    def render_high(self, d, sync: bool = True) -> None:
        self.high.update(sc.orbit_view(self.s, d, 2 * self.width, 2 * self.height))
        _render(self.high, sync)

    def high_color(self) -> int:
        return int(self.high.frame().color_rgba8)

    def close(self) -> None:
        self.low.deinit()
        self.high.deinit()


def _stream_sync(stream: int) -> None:
    import torch

    torch.cuda.ExternalStream(stream).synchronize()


def train(steps: int = 3000, batch: int = 4, lr: float = 2e-3, seed: int = 0, scene_seed: int = 0,
          width: int = 960, height: int = 540, log=print, samples: int = 1) -> tuple[np.ndarray, list]:
    """Adam on the loss sum over `batch` frames per step (cosine learning-rate decay);
    returns the parameters and the per-step mean squared error."""
    s = sc.random_triangles(seed=scene_seed, width=2 * width, height=2 * height)
    pr = PairRenderer(s, width, height, samples=samples)
    u = Upsampler(0, width, height)
    u.set_params(init_params(seed))
    dirs = sc.camera_dirs(TRAIN_CAMERAS, TRAIN_CAMERA_SEED)
    rng = np.random.Generator(np.random.PCG64(seed))
    stream = pr.low.stream
    hist = []
    t0 = time.perf_counter()
    for step in range(steps):
        lr_t = lr * 0.5 * (1.0 + math.cos(math.pi * step / steps))
        for _ in range(batch):
            d = dirs[int(rng.integers(TRAIN_CAMERAS))]
            pr.render_high(d)
            pr.render_low(d)
            u.accumulate(pr.low.gbuffer(), pr.high_color(), None, stream)
            _stream_sync(stream)  # the next frames overwrite both renderers' buffers
        loss, values = u.loss(stream)
        hist.append(loss / values)
        u.adam_step(lr_t, grad_scale=1.0 / values, stream=stream)
        if log and (step % 100 == 0 or step == steps - 1):
            mse = hist[-1]
            log(f"step {step:5d}  mse {mse:.3e}  ({10 * math.log10(1.0 / max(mse, 1e-30)):.2f} dB)  lr {lr_t:.2e}  "
                f"{time.perf_counter() - t0:.1f} s")
    if u.status() != 0:
        raise RuntimeError("upsampler kernels reported an error")
    p = u.params()
    u.close()
    pr.close()
    return p, hist


def _psnr_dev(a, b) -> tuple[float, int]:
    """PSNR (dB) and max abs error of the RGB bytes of two (H, W, 4) uint8 device tensors."""
    d = (a[..., :3].int() - b[..., :3].int())
    mse = float((d.float() ** 2).mean().item())
    mx = int(d.abs().max().item())
    return (float("inf") if mse == 0 else 10.0 * math.log10(255.0 ** 2 / mse)), mx


def evaluate(params: np.ndarray, cameras: int = TEST_CAMERAS, scene_seed: int = 0, width: int = 960,
             height: int = 540, samples: int = 1) -> dict:
    """Per held-out frame, against the plain full-resolution render: PSNR and max
    error of the learned reconstruction, of the x2 base alone (the network's
    parameters zero: the triangle-aware base where the G-buffer has sub-pixel
    sources) and of plain bilinear upsampling (the base without sources)."""
    import torch

    from .graphics import _DeviceView

    s = sc.random_triangles(seed=scene_seed, width=2 * width, height=2 * height)
    pr = PairRenderer(s, width, height, samples=samples)
    net = Upsampler(0, width, height)
    net.set_params(params)
    zero = Upsampler(0, width, height)
    zero.set_params(np.zeros(PARAM_COUNT, np.float32))
    out_n = torch.zeros((2 * height, 2 * width), dtype=torch.int32, device="cuda")
    out_z = torch.zeros_like(out_n)
    out_b = torch.zeros_like(out_n)
    dirs = sc.camera_dirs(cameras, TEST_CAMERA_SEED)
    stream = pr.low.stream
    frames = []

    def img(t):
        return t.view(torch.uint8).view(2 * height, 2 * width, 4)

    for d in dirs:
        pr.render_high(d)
        pr.render_low(d)
        gb = pr.low.gbuffer()
        net.infer(gb, out_n.data_ptr(), stream)
        zero.infer(gb, out_z.data_ptr(), stream)
        gb.sources_u16 = None
        zero.infer(gb, out_b.data_ptr(), stream)
        _stream_sync(stream)
        f = pr.high.frame()
        ref = torch.as_tensor(_DeviceView(f.color_rgba8, (2 * height, 2 * width, 4), "|u1"), device="cuda")
        pn, mn = _psnr_dev(img(out_n), ref)
        pz, mz = _psnr_dev(img(out_z), ref)
        pb, mb = _psnr_dev(img(out_b), ref)
        frames.append({"psnr_db": pn, "max_abs_error": mn, "base_psnr_db": pz, "base_max_abs_error": mz,
                       "bilinear_psnr_db": pb, "bilinear_max_abs_error": mb})
    net.close()
    zero.close()
    pr.close()
    pn = [f["psnr_db"] for f in frames]
    pz = [f["base_psnr_db"] for f in frames]
    pb = [f["bilinear_psnr_db"] for f in frames]
    return {
        "frames": len(frames), "psnr_db_mean": float(np.mean(pn)), "psnr_db_min": float(np.min(pn)),
        "psnr_db_median": float(np.median(pn)), "max_abs_error": int(max(f["max_abs_error"] for f in frames)),
        "frames_at_or_above_floor": int(sum(p >= PSNR_FLOOR_DB for p in pn)),
        "base_psnr_db_mean": float(np.mean(pz)), "base_psnr_db_min": float(np.min(pz)),
        "base_frames_at_or_above_floor": int(sum(p >= PSNR_FLOOR_DB for p in pz)),
        "bilinear_psnr_db_mean": float(np.mean(pb)), "bilinear_psnr_db_min": float(np.min(pb)),
        "bilinear_max_abs_error": int(max(f["bilinear_max_abs_error"] for f in frames)),
        "per_frame": frames,
    }


def time_paths(params: np.ndarray, frames: int = 64, warmup: int = 5, scene_seed: int = 0, width: int = 960,
               height: int = 540, samples: int = 1) -> dict:
    """Device time per frame of the plain 2W x 2H path and of the learned path (W x H render +
    upsampler), each frame after a 256 MiB L2 flush, cycling the held-out cameras; and the
    upsampler alone."""
    import torch

    s = sc.random_triangles(seed=scene_seed, width=2 * width, height=2 * height)
    pr = PairRenderer(s, width, height, samples=samples)
    net = Upsampler(0, width, height)
    net.set_params(params)
    out = torch.zeros((2 * height, 2 * width), dtype=torch.int32, device="cuda")
    dirs = sc.camera_dirs(TEST_CAMERAS, TEST_CAMERA_SEED)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for i in range(warmup):  # grows the raster queues, builds the graphs
        pr.render_high(dirs[i])
        pr.render_low(dirs[i])
        net.infer(pr.low.gbuffer(), out.data_ptr(), pr.low.stream)
    _stream_sync(pr.low.stream)

    def run(kind):
        st = torch.cuda.ExternalStream(pr.high.stream if kind == "plain" else pr.low.stream)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(frames)]
        with torch.cuda.stream(st):
            for i in range(frames):
                flush.fill_(float(i))
                d = dirs[i % len(dirs)]
                ev[i][0].record(st)
                if kind == "plain":
                    pr.render_high(d, sync=False)
                elif kind == "learned":
                    pr.render_low(d, sync=False)
                    net.infer(pr.low.gbuffer(), out.data_ptr(), pr.low.stream)
                else:  # the network alone on the last G-buffer
                    net.infer(pr.low.gbuffer(), out.data_ptr(), pr.low.stream)
                ev[i][1].record(st)
        st.synchronize()
        return float(np.mean([a.elapsed_time(b) for a, b in ev]))

    plain = run("plain")
    learned = run("learned")
    net_ms = run("net")
    if net.status() != 0:
        raise RuntimeError("upsampler kernels reported an error")
    net.close()
    pr.close()
    flops = conv_flops(width, height, real_channels=True, real_in=14 if samples == 1 else 10)
    return {
        "plain_ms": plain, "plain_fps": 1e3 / plain, "learned_ms": learned, "learned_fps": 1e3 / learned,
        "speedup": plain / learned, "upsampler_ms": net_ms,
        "upsampler_tflops": flops / (net_ms * 1e-3) / 1e12, "upsampler_flops": flops,
        "triangles": s.triangle_count, "frames": frames,
    }


def load_weights(path: str = WEIGHTS) -> tuple[np.ndarray, dict]:
    z = np.load(path, allow_pickle=False)
    meta = json.loads(str(z["meta"])) if "meta" in z else {}
    return z["params"].astype(np.float32), meta


class LearnedPath:
    """Renders 2W x 2H frames through the learned path, or through the plain path
    (the fallback) unless the plain render, judging each held-out frame, found
    every one of them at or above the floor: `heldout_psnr_db` is the list of
    per-frame PSNRs from `evaluate` (a single number is taken as the minimum)."""

    def __init__(self, s: sc.Scene, width: int, height: int, params: np.ndarray, heldout_psnr_db,
                 samples: int = 1):
        import torch

        self.pr = PairRenderer(s, width, height, samples=samples)
        self.net = Upsampler(0, width, height)
        self.net.set_params(params)
        worst = float(np.min(np.asarray(heldout_psnr_db, np.float64)))
        self.use_network = worst >= PSNR_FLOOR_DB
        self.out = torch.zeros((2 * height, 2 * width), dtype=torch.int32, device="cuda")

    def render(self, cam_dir) -> int:
        """Device pointer of the RGBA8 2W x 2H frame for camera direction `cam_dir` (valid
        until the next call; synchronised)."""
        if not self.use_network:
            self.pr.render_high(cam_dir)
            return self.pr.high_color()
        self.pr.render_low(cam_dir)
        self.net.infer(self.pr.low.gbuffer(), self.out.data_ptr(), self.pr.low.stream)
        _stream_sync(self.pr.low.stream)
        return self.out.data_ptr()

    def close(self) -> None:
        self.net.close()
        self.pr.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "eval", "time"])
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cameras", type=int, default=TEST_CAMERAS)
    ap.add_argument("--samples", type=int, default=1, choices=[1, 4])
    ap.add_argument("--weights", default=None)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    default = WEIGHTS if args.samples == 1 else WEIGHTS_MSAA4
    args.weights = args.weights or default
    args.out = args.out or default
    from . import build

    build.build()
    if args.cmd == "train":
        t0 = time.perf_counter()
        p, hist = train(args.steps, args.batch, args.lr, args.seed, samples=args.samples)
        ev = evaluate(p, args.cameras, samples=args.samples)
        meta = {"steps": args.steps, "batch": args.batch, "lr": args.lr, "seed": args.seed, "samples": args.samples,
                "inputs": "colour, albedo, normal, coverage, depth" + (", sub-pixel sources" if args.samples == 1 else ""),
                "train_cameras": TRAIN_CAMERAS, "train_camera_seed": TRAIN_CAMERA_SEED,
                "test_cameras": args.cameras, "test_camera_seed": TEST_CAMERA_SEED,
                "final_train_mse": float(np.mean(hist[-50:])), "train_seconds": time.perf_counter() - t0,
                "heldout": {k: v for k, v in ev.items() if k != "per_frame"}}
        os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
        np.savez(args.out, params=p, meta=json.dumps(meta), train_mse=np.asarray(hist, np.float32))
        print(json.dumps(meta))
    elif args.cmd == "eval":
        p, _ = load_weights(args.weights)
        ev = evaluate(p, args.cameras, samples=args.samples)
        print(json.dumps({k: v for k, v in ev.items() if k != "per_frame"}))
    else:
        p, _ = load_weights(args.weights)
        print(json.dumps(time_paths(p, samples=args.samples)))


if __name__ == "__main__":
    main()
