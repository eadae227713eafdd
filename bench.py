"""Frame-rate benchmark of the GB300 renderer (shadow pass + camera pass + shading).

Workload (default): the scene-scale configuration — 64 meshes totalling 262,144
triangles, 32 materials with 1024^2 albedo/normal/metal-roughness textures and
full mips, a 4096^2 D32 shadow map with 3x3 PCF, 1920x1080 output, 8 camera
frames along a seeded Catmull-Rom spline (seed 0). Synthetic, seeded inputs.

A step is one frame (camera i mod 8). `value` is frames/s over the device time
of the frames (CUDA events on the renderer's stream; the scene constants are
uploaded inside the frame, everything else is resident); L2 is flushed by a
256 MiB write between frames, outside the timed events. `e2e` is frames/s
through the C ABI with host buffers: per frame, the scene constants and all
object transforms go host->device from pinned memory and the RGBA8 frame comes
back device->host into pinned memory (copied straight from the frame's target
set on the renderer's copy stream while the next frame renders into the other),
wall-clock timed, with two frames in flight (a host buffer is reused once the
read-back that last filled it has landed, rz_read_sync;
the reference's Vulkan renderer keeps up to three, src/Engine/Graphics.cpp:177).

--impl reference times the CPU restatement of the reference's path (the oracle,
oracle/rz_oracle.cpp; Rosy itself needs Vulkan on Windows and cannot run here)
on all host threads, on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "1080p frames/s/GPU (plain path)"
UNIT = "frames/s"
L2_FLUSH_BYTES = 256 << 20


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["bf16_tflops"]), "measured (MEASURED_PEAKS.json bf16_tflops, burst)"
    return 1900.0, "fallback 1.9 PFLOP/s"


def learned_block(frames: int = 64, cameras: int = 256, samples: int = 1) -> dict:
    """The learned half-resolution path against the plain path at 1920x1080 on the
    random-triangles scene: device frames/s of both, held-out PSNR and max error per
    frame against the plain render, and the upsampler's tensor-core roofline. With
    samples = 4 both renders use the reference's 4x multisampling (and the network
    trained on such frames)."""
    from rosy_gb300 import learned

    params, meta = learned.load_weights(learned.WEIGHTS if samples == 1 else learned.WEIGHTS_MSAA4)
    t = learned.time_paths(params, frames=frames, samples=samples)
    ev = learned.evaluate(params, cameras, samples=samples)
    peak, src = bf16_peak()
    per = ev.pop("per_frame")
    up_in = 14 if samples == 1 else 10  # real input channels: the sub-pixel sources exist single-sampled
    return {
        "workload": "random_triangles (4,096 triangles, 256^2 texture, 1024^2 shadow map): plain 1920x1080 vs "
                    "960x540 render + upsampler to 1920x1080; L2 flushed between frames",
        "samples_per_pixel": samples,
        "plain_fps": round(t["plain_fps"], 2), "learned_fps": round(t["learned_fps"], 2),
        "speedup": round(t["speedup"], 3), "plain_ms": round(t["plain_ms"], 5), "learned_ms": round(t["learned_ms"], 5),
        "heldout": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in ev.items()},
        "psnr_floor_db": learned.PSNR_FLOOR_DB,
        "frames_below_floor": ev["frames"] - ev["frames_at_or_above_floor"],
        "fallback_to_plain": ev["frames_at_or_above_floor"] < ev["frames"],  # judged per held-out frame
        "per_frame_psnr_db": [round(f["psnr_db"], 2) for f in per],
        "per_frame_max_abs_error": [f["max_abs_error"] for f in per],
        "per_frame_base_psnr_db": [round(f["base_psnr_db"], 2) for f in per],
        "upsampler_roofline": {"bound": "tensor", "achieved": round(t["upsampler_tflops"], 2), "peak": peak,
                               "unit": "TFLOP/s", "frac": round(t["upsampler_tflops"] / peak, 4),
                               "peak_source": src, "ms_per_frame": round(t["upsampler_ms"], 5),
                               "flops_per_frame": t["upsampler_flops"],
                               "flops_note": "2 x 9 x cin x cout x 960 x 540 over the real channels "
                                             f"({up_in}-32-32-32-12)"},
        "weights": {k: meta.get(k) for k in ("steps", "batch", "lr", "train_cameras", "train_seconds", "inputs")},
    }


def bc7_block(size: int = 8192, reps: int = 10) -> dict:
    """BC7 decode (rz_bc7_decode, the upload-time decode of the reference's BC7
    images) of one size x size image whose blocks cycle through every mode:
    device time per decode with the L2 flushed between decodes, the HBM roofline
    over the algorithmic bytes (16 read + 64 written per 4x4 block), and the
    scalar oracle's decode rate on one host core for comparison."""
    import ctypes as C

    import torch

    from oracle import oracle
    from rosy_gb300 import _lib, bc7

    lib = _lib.load()
    rng = np.random.default_rng(11)
    base = bc7.mixed_blocks(rng, 4096)
    nblk = (size // 4) ** 2
    blocks = torch.from_numpy(base[rng.integers(0, len(base), nblk)].reshape(-1)).cuda()
    out = torch.empty(size * size, dtype=torch.int32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    for _ in range(3):
        assert lib.rz_bc7_decode(C.c_void_p(blocks.data_ptr()), size, size, C.c_void_p(out.data_ptr()), sp) == 0
    times = []
    for _ in range(reps):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        lib.rz_bc7_decode(C.c_void_p(blocks.data_ptr()), size, size, C.c_void_p(out.data_ptr()), sp)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    ms = float(np.median(times))
    algo = nblk * (16 + 64)
    peak, src = peaks()
    gbs = algo / (ms * 1e-3) / 1e9
    # the oracle on one core, a 512 x 512 sample of the same blocks
    host = blocks[: (128 * 128) * 16].cpu().numpy()
    t0 = time.perf_counter()
    oracle.bc7_decode(host, 512, 512)
    cpu_s = time.perf_counter() - t0
    return {
        "workload": f"{size}x{size} texels ({nblk} BC7 blocks, modes 0-7 cycling), L2 flushed between decodes",
        "ms": round(ms, 5), "gtexels_per_s": round(size * size / (ms * 1e-3) / 1e9, 2),
        "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(gbs / peak, 4), "peak_source": src,
                     "algorithmic_bytes": algo, "bytes_note": "16 B read + 64 B written per block"},
        "cpu_oracle": {"mtexels_per_s": round(512 * 512 / cpu_s / 1e6, 2), "cores": 1,
                       "sample": "512x512 texels of the same blocks, scalar oracle"},
    }


def measured_traffic(stage: str):
    """DRAM bytes per launch of a kernel from the committed ncu summary of this
    workload (profiles/dram_traffic_scene_scale_1080p.json), or None."""
    p = os.path.join(ROOT, "profiles", "dram_traffic_scene_scale_1080p.json")
    try:
        return json.load(open(p))["dram_bytes_per_launch"].get(stage)
    except (OSError, ValueError, KeyError):
        return None


def make_scene(name: str, samples: int = 1):
    from rosy_gb300 import scene as sc

    if name == "scene_scale":
        s = sc.scene_scale(seed=0)
        s.samples = samples
        return s
    if name == "random_triangles":
        s = sc.random_triangles(seed=0)
        s.samples = samples
        return s
    raise SystemExit(f"unknown config {name}")


def workload_config(name: str, s) -> dict:
    return {
        "workload": name, "triangles": s.triangle_count, "meshes": len(s.meshes),
        "materials": len(s.materials), "textures": len(s.textures),
        "texture_size": s.textures[0].width if s.textures else 0,
        "width": s.width, "height": s.height, "shadow_map": s.shadow_size,
        "pcf": "3x3" if int(s.draw_config["pcf_mode"][0]) == 1 else "5-tap",
        "frames_on_spline": len(s.cameras), "seed": 0, "samples_per_pixel": getattr(s, "samples", 1),
        "l2": "flushed between frames (256 MiB write)",
    }


class Clocks:
    """Samples nvidia-smi during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        import tempfile

        self.path = tempfile.mktemp(suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(int(os.environ.get("LOCAL_RANK", "0")))],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for i, n in enumerate(names):
                if r[5 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if os.environ.get("RZ_BENCH_BACKEND") != "gloo" else "gloo")
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(s, seconds: float) -> tuple[dict, dict]:
    """Times the CPU restatement on a bounded sample: whole frames of the same
    workload, as many as fit in `seconds` (at least one)."""
    from oracle import oracle

    threads = os.cpu_count() or 1
    oracle.build()
    t0 = time.perf_counter()
    n = 0
    while True:
        oracle.render(s.with_camera(n), threads=threads)
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    # the same restatement on one host thread: one frame
    t1 = time.perf_counter()
    oracle.render(s.with_camera(0), threads=1)
    dt1 = time.perf_counter() - t1
    extra = {}
    r = oracle.render(s.with_camera(0), threads=threads, texel_bytes=True, fp64=True)
    extra["texel_bytes"] = r["texel_bytes"]
    extra["oracle_ids"] = r["ids"]
    extra["oracle_color"] = r["color"]
    extra["oracle_color_f64"] = r["color_f64"]
    return ({"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
             "sample": f"{n} full frame(s) of the same workload (spline cameras cycled), {dt:.1f} s",
             "single_thread": {"value": round(1.0 / dt1, 4), "unit": UNIT, "cores": 1,
                               "sample": f"1 full frame (camera 0), {dt1:.2f} s"}}, extra)


def shade_bytes(s, ids: np.ndarray, texel_bytes: int | None) -> int | None:
    """Algorithmic bytes of the shading kernel: visibility read, RGBA8 + D32 out,
    the vertices of the visible triangles, materials, and the compulsory texels."""
    if texel_bytes is None:
        return None
    W, H = s.width, s.height
    vis = ids[ids > 0].astype(np.int64) - 1
    # opaque list == all surfaces here; map triangle ids to vertex indices
    surf = s.surfaces
    counts = (surf["index_count"] // 3).astype(np.int64)
    base = np.concatenate([[0], np.cumsum(counts)])
    tri = np.unique(vis)
    d = np.searchsorted(base, tri, side="right") - 1
    mesh = surf["mesh_index"][d]
    mt = np.asarray(s.meshes, np.int64)
    first = mt[mesh, 2] + surf["start_index"][d].astype(np.int64) + 3 * (tri - base[d])
    verts = np.unique(np.concatenate([s.indices[first + k].astype(np.int64) + mt[mesh, 0] for k in range(3)]))
    ns = getattr(s, "samples", 1)
    return 8 * W * H * ns + 4 * W * H + 4 * W * H + 64 * len(verts) + 64 * len(s.materials) + int(texel_bytes)


def raster_bytes(s, pass_name: str) -> int:
    """Algorithmic bytes of a raster pass: vertex pull once, indices, objects, target write."""
    V = len(s.vertices)
    T = s.triangle_count
    D = len(s.surfaces)
    if pass_name == "shadow":
        return 64 * V + 12 * T + 164 * D + 4 * s.shadow_size ** 2
    return 64 * V + 12 * T + 164 * D + 8 * s.width * s.height * getattr(s, "samples", 1)


def run_rz(args):
    import torch

    rank, ws = dist_init()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from rosy_gb300 import build as rzbuild

    rzbuild.build()
    from rosy_gb300.graphics import Graphics

    s = make_scene(args.config, args.samples)
    g = Graphics()
    g.init(s.width, s.height, s.shadow_size, device=torch.cuda.current_device(), samples=s.samples)
    g.set_asset(s)
    g.set_graphic_objects(s.objects, s.surfaces)
    g.set_draw_config(s.draw_config)
    stream = torch.cuda.ExternalStream(g.stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    cams = [np.ascontiguousarray(c) for c in s.cameras]

    for i in range(args.warmup):
        g.update(cams[i % len(cams)])
        g.render()
    g.sync()
    # the renderer's autotuner picks the work-chunk size and small-triangle extent
    # for this workload (it renders the current frame with each candidate), then
    # the chosen tuning is warmed up like the first
    tuned, tune_ms = g.autotune(frames=3)
    for i in range(args.warmup):
        g.update(cams[i % len(cams)])
        g.render()
    g.sync()

    # --- timed region: device time of each frame ---
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = Clocks()
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(float(i))
            starts[i].record(stream)
            g.update(cams[i % len(cams)])
            g.render()
            ends[i].record(stream)
    g.sync()
    torch.cuda.synchronize()
    barrier(ws)
    ck = clocks.stop()
    frame_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = max_over_ranks(sum(frame_ms), ws)
    value = ws * args.steps / (total_ms / 1e3)
    if args.profile:  # short run for ncu: the timed frames only
        g.deinit()
        if rank == 0:
            print(json.dumps({"profile_run": True, "frames_per_s": round(value, 2)}))
        return

    # --- per-stage times (same frames, stage events on) ---
    g.set_stage_timing(True)
    stage_acc = {}
    n_stage = min(args.steps, 200)
    for i in range(n_stage):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        g.update(cams[i % len(cams)])
        g.render()
        g.sync()
        for k, v in g.stage_times().items():
            stage_acc[k] = stage_acc.get(k, 0.0) + v
    stage_ms = {k: v / n_stage for k, v in stage_acc.items()}
    g.set_stage_timing(False)
    g.render()  # back to the graph path
    g.sync()
    stats = g.stats()

    # --- e2e through the C ABI with host buffers, two frames in flight ---
    ring = 2
    color_hosts = [torch.empty((s.height, s.width, 4), dtype=torch.uint8, pin_memory=True).numpy()
                   for _ in range(ring)]
    objects_host = torch.empty(s.objects.shape, dtype=torch.float32, pin_memory=True).numpy()
    objects_host[:] = s.objects
    scene_host = [torch.empty(408, dtype=torch.uint8, pin_memory=True).numpy() for _ in cams]
    for k, c in enumerate(cams):
        scene_host[k][:] = np.frombuffer(c.tobytes(), np.uint8)
    n_e2e = min(args.steps, 200)
    # the C ABI called directly with arguments prepared once (the wrappers' checks and
    # numpy conversions would otherwise be timed as part of every frame)
    lib, ctx = g._lib, g._ctx
    scene_ptrs = [h.ctypes.data for h in scene_host]
    obj_ptr, n_obj = objects_host.ctypes.data, len(objects_host)
    color_ptrs = [h.ctypes.data for h in color_hosts]
    color_bytes = color_hosts[0].nbytes
    g.sync()
    barrier(ws)
    rcs = 0
    t0 = time.perf_counter()
    for i in range(n_e2e):
        k = i % ring
        if i >= ring:
            rcs |= lib.rz_read_sync(ctx, 1, 0)  # every read-back but the newest has landed: this buffer is free
        rcs |= lib.rz_update(ctx, scene_ptrs[i % len(cams)])
        rcs |= lib.rz_update_objects(ctx, 0, obj_ptr, n_obj)
        rcs |= lib.rz_render(ctx)
        rcs |= lib.rz_read_frame(ctx, color_ptrs[k], color_bytes, None, 0)
    g.sync()
    if rcs:
        raise RuntimeError(f"e2e loop: a C ABI call failed ({g._lib.rz_last_error(g._ctx)})")
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    e2e_value = ws * n_e2e / e2e_s

    # --- roofline of the dominant kernel ---
    hbm, peak_kind = peaks()
    dominant = max(stage_ms, key=stage_ms.get)
    cpu = None
    extra = {}
    if rank == 0 and not args.no_cpu_baseline:
        cpu, extra = cpu_baseline(s, args.cpu_seconds)
    g.update(cams[0])
    g.render()
    g.sync()
    out0 = g.download() if rank == 0 else None
    algo = {
        "shadow_raster": raster_bytes(s, "shadow"),
        "camera_raster": raster_bytes(s, "camera"),
        "shade": shade_bytes(s, out0["ids"], extra.get("texel_bytes")) if out0 is not None else None,
        # a setup launch pulls the vertices, indices and objects and zeroes its pass's depth
        # target: the same byte count as its raster launch (which reads the setup records and
        # writes that target). The clear stages before them only reset pass headers.
        "shadow_setup": raster_bytes(s, "shadow"),
        "camera_setup": raster_bytes(s, "camera"),
    }
    roof = None
    if rank == 0:
        stage = dominant
        b = algo.get(stage)
        if b is None:  # no algorithmic byte count for this stage: report the shading kernel
            stage = "shade"
            b = algo["shade"]
        if b is not None:
            ach = b / (stage_ms[stage] / 1e3) / 1e9
            roof = {"kernel": stage, "bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(ach / hbm, 4), "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                    if peak_kind == "measured" else "fallback 6.8 TB/s",
                    "algorithmic_bytes_per_launch": int(b), "ms_per_launch": round(stage_ms[stage], 5),
                    "traffic": measured_traffic(stage) if args.config == "scene_scale" else None,
                    "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                      "profiles/dram_traffic_scene_scale_1080p.json"}
    by_stage = {}  # every stage with an algorithmic byte count (the shading pass and the shadow raster are close)
    for st, b in algo.items():
        if rank == 0 and b is not None and stage_ms.get(st):
            ach = b / (stage_ms[st] / 1e3) / 1e9
            by_stage[st] = {"achieved_gbs": round(ach, 1), "frac": round(ach / hbm, 4), "ms": round(stage_ms[st], 5),
                            "algorithmic_bytes": int(b)}
    parity = None
    fp64 = None
    if rank == 0 and extra.get("oracle_ids") is not None:
        parity = bool(np.array_equal(out0["ids"], extra["oracle_ids"]))
        # shading error against the oracle evaluated in float64 (sRGB value * 255, before 8-bit rounding)
        ref = extra["oracle_color_f64"][..., :3] * 255.0
        e_gpu = np.abs(out0["color"][..., :3].astype(np.float64) - ref)
        e_o32 = np.abs(extra["oracle_color"][..., :3].astype(np.float64) - ref)
        d32 = np.abs(out0["color"][..., :3].astype(np.int32) - extra["oracle_color"][..., :3].astype(np.int32))
        fp64 = {"frame": 0, "unit": "1/255 of the sRGB value",
                "gpu_max_abs": round(float(e_gpu.max()), 4), "gpu_mean_abs": round(float(e_gpu.mean()), 4),
                "oracle_fp32_max_abs": round(float(e_o32.max()), 4),
                "oracle_fp32_mean_abs": round(float(e_o32.mean()), 4),
                "gpu_vs_oracle_fp32_max_levels": int(d32.max()),
                "note": "8-bit rounding alone contributes up to 0.5"}
    g.deinit()
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": workload_config(args.config, s),
            "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": 408 + int(s.objects.nbytes),
                    "d2h_bytes_per_step": int(s.width * s.height * 4), "steps": n_e2e, "frames_in_flight": ring},
            "gpu_launches": int(stats.kernel_launches) * args.steps,
            "tuning": {"autotuned": tuned, "candidates_ms": [round(x, 4) for x in tune_ms]},
            "raster_work": {"shadow_records": int(stats.shadow_setup_records), "shadow_stamps": int(stats.shadow_stamps),
                            "camera_records": int(stats.camera_setup_records), "camera_stamps": int(stats.camera_stamps)},
            "roofline": roof,
            "roofline_by_stage": by_stage,
            "stage_ms": {k: round(v, 5) for k, v in stage_ms.items()},
            "mtriangles_per_s": round(value * s.triangle_count / 1e6, 1),
            "cpu_baseline": cpu,
            "clocks": ck,
            "visibility_matches_oracle_frame0": parity,
            "fp64_oracle_error": fp64,
            "algorithmic_bytes": {k: (int(v) if v is not None else None) for k, v in algo.items()},
        }
        if not args.no_learned:
            line["learned_upsample"] = learned_block()
            line["learned_upsample_msaa4"] = learned_block(samples=4)
        line["bc7_decode"] = bc7_block()
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_batch(args):
    """Batched views: 256 views of log-uniform extent 64..1024 over 16 scenes of
    1k-200k triangles, each view with its own 512..2048 shadow map. One rz_render
    renders all views (one launch per stage, one CUDA graph); compared with the
    same kernels launched view by view. The autotuner picks the work-chunk size
    and the small-triangle extent first."""
    import torch

    from rosy_gb300 import build as rzbuild
    from rosy_gb300 import scene as sc

    from rosy_gb300.replicas import shard_range

    rank, ws = dist_init()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rzbuild.build()
    from rosy_gb300.graphics import Graphics

    scenes, all_views = sc.batch_views(seed=0, views=args.views, scenes=16)
    vb, ve = shard_range(len(all_views), rank, ws)
    views = all_views[vb:ve]
    g = Graphics()
    g.init(64, 64, 64, device=torch.cuda.current_device())
    idx = [g.add_scene(s) for s in scenes]
    g.set_views([(idx[k], v.width, v.height, v.shadow_size, v.draw_config) for k, v in views])
    for i, (_, v) in enumerate(views):
        g.update_view(i, v.scene)
    for _ in range(2):
        g.render()
        g.sync_code()
    tuned, cand_ms = g.autotune(frames=3)
    stream = torch.cuda.ExternalStream(g.stream)

    def timed(steps):
        for _ in range(args.warmup):
            g.render()
        g.sync()
        barrier(ws)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            g.render()
        b.record(stream)
        g.sync()
        barrier(ws)
        return max_over_ranks(a.elapsed_time(b) / steps, ws)

    steps = max(3, min(args.steps, 50))
    batched_ms = timed(steps)
    g.set_tuning(tuned["chunk_stamps"], tuned["small_extent"], 0, batched=False)
    seq_ms = timed(max(3, steps // 5))
    g.deinit()
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    if rank != 0:
        return
    px = sum(v.width * v.height for _, v in all_views)
    tris = sum(scenes[k].triangle_count for k, _ in all_views)
    print(json.dumps({
        "metric": f"batched views: views/s ({len(all_views)} views, {len(scenes)} scenes)",
        "value": round(len(all_views) / (batched_ms / 1e3), 1),
        "unit": "views/s", "n_gpus": ws, "steps": steps, "warmup": args.warmup, "ms_per_step": round(batched_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": "batch_views", "views": len(all_views), "scenes": len(scenes),
                   "views_per_rank": "contiguous shards" if ws > 1 else len(all_views),
                   "pixels_per_batch": px, "triangles_per_batch_per_pass": tris,
                   "shadow_texels_per_batch": sum(v.shadow_size ** 2 for _, v in views)},
        "sequential_ms_per_batch": round(seq_ms, 4), "batched_speedup_vs_sequential": round(seq_ms / batched_ms, 3),
        "autotuned": tuned, "autotune_candidates_ms": [round(x, 4) for x in cand_ms],
    }))


def run_stress(args):
    """The combined stress workload (1,048,576 triangles, 256 meshes, 64 materials with
    2048^2 textures, 4 shadow cascades of 4096^2, 3x3 PCF): a batch of 8 views along
    the camera spline rendered at 3840x2160 by the plain path, against the same 8 views
    rendered at 1920x1080 (G-buffer on) and upsampled to 3840x2160 by the learned
    upsampler. Reports views/s of both, per-view PSNR and max error of the learned
    views against the plain ones."""
    import torch

    from rosy_gb300 import build as rzbuild
    from rosy_gb300 import learned
    from rosy_gb300 import scene as sc
    from rosy_gb300.upsampler import Upsampler, psnr

    rzbuild.build()
    from rosy_gb300.graphics import Graphics

    views = 8
    s = sc.stress(frames=views)
    lo_recs = [sc.view_of(s, 1920, 1080, 4096, camera=i).scene for i in range(views)]
    params, meta = learned.load_weights(learned.WEIGHTS if args.samples == 1 else learned.WEIGHTS_MSAA4)

    def ctx(w, h, gbuffer):
        g = Graphics()
        g.init(w, h, 4096, samples=args.samples)
        g.set_asset(s)
        g.set_graphic_objects(s.objects, s.surfaces)
        g.set_draw_config(s.draw_config)
        g.set_views([(0, w, h, 4096, s.draw_config)] * views)
        if gbuffer:
            g.set_gbuffer(True)
        return g

    plain = ctx(3840, 2160, False)
    for i in range(views):
        plain.update_view(i, s.cameras[i])
    low = ctx(1920, 1080, True)
    for i in range(views):
        low.update_view(i, lo_recs[i])
    net = Upsampler(0, 1920, 1080)
    net.set_params(params)
    outs = [torch.zeros((2160, 3840), dtype=torch.int32, device="cuda") for _ in range(views)]
    for g in (plain, low):  # grow the queues, build the graphs
        for _ in range(3):
            g.render()
            if g.sync_code() != 14:
                break
        g.sync()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def timed(kind, steps):
        g = plain if kind == "plain" else low
        st = torch.cuda.ExternalStream(g.stream)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(st):
            for i in range(steps + args.warmup):
                flush.fill_(float(i))
                if i >= args.warmup:
                    ev[i - args.warmup][0].record(st)
                g.render()
                if kind == "learned":
                    for v in range(views):
                        net.infer(low.gbuffer(v), outs[v].data_ptr(), low.stream)
                if i >= args.warmup:
                    ev[i - args.warmup][1].record(st)
        st.synchronize()
        return float(np.mean([a.elapsed_time(b) for a, b in ev]))

    steps = max(3, min(args.steps, 20))
    plain_ms = timed("plain", steps)
    learned_ms = timed("learned", steps)
    per = []
    for v in range(views):
        ref = plain.download_view(v)["color"]
        got = outs[v].cpu().numpy().view(np.uint8).reshape(2160, 3840, 4)
        d = np.abs(got[..., :3].astype(np.int32) - ref[..., :3].astype(np.int32))
        per.append({"psnr_db": round(psnr(got, ref), 3), "max_abs_error": int(d.max())})
    if net.status() != 0:
        raise RuntimeError("upsampler kernels reported an error")
    net.close()
    plain.deinit()
    low.deinit()
    print(json.dumps({
        "metric": "stress: 3840x2160 views/s, plain vs 1920x1080 + learned upsampler", "unit": "views/s",
        "value": round(views / (learned_ms / 1e3), 2), "plain_value": round(views / (plain_ms / 1e3), 2),
        "speedup": round(plain_ms / learned_ms, 3), "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_batch": {"plain": round(plain_ms, 4), "learned": round(learned_ms, 4)},
        "higher_is_better": True, "dtype": "f32 raster/shading, bf16 upsampler", "data": "synthetic (seeded)",
        "config": {"workload": "stress", "samples_per_pixel": args.samples, "triangles": s.triangle_count,
                   "meshes": 256, "materials": 64,
                   "textures": len(s.textures), "texture_size": 2048, "shadow_cascades": 4, "shadow_map": 4096,
                   "views_per_batch": views, "plain_extent": [3840, 2160], "render_extent": [1920, 1080],
                   "l2": "flushed between batches (256 MiB write)"},
        "per_view": per, "psnr_db_mean": round(float(np.mean([p["psnr_db"] for p in per])), 3),
        "psnr_floor_db": learned.PSNR_FLOOR_DB,
        "fallback_to_plain": any(p["psnr_db"] < learned.PSNR_FLOOR_DB for p in per),  # judged per view
        "weights": {k: meta.get(k) for k in ("steps", "train_cameras")},
    }))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    s = make_scene(args.config, args.samples)
    from oracle import oracle

    oracle.build()
    threads = os.cpu_count() or 1
    # the requested warm-up frames, untimed (capped at the sample's time budget)
    warm = 0
    tw = time.perf_counter()
    while warm < args.warmup and time.perf_counter() - tw < args.cpu_seconds:
        oracle.render(s.with_camera(warm), threads=threads)
        warm += 1
    t0 = time.perf_counter()
    n = 0
    while n < args.steps:
        oracle.render(s.with_camera(n), threads=threads)
        n += 1
        if time.perf_counter() - t0 >= args.cpu_seconds:
            break
    dt = time.perf_counter() - t0
    v = n / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": 1, "steps": n,
        "warmup": warm, "ms_per_step": round(1e3 * dt / n, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": workload_config(args.config, s),
        "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} full frame(s), capped at {args.cpu_seconds:.0f} s"},
        "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference (Vulkan, Windows-only) cannot run here; its path is timed as the scalar CPU "
                "restatement in oracle/rz_oracle.cpp on all host threads",
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="rz", choices=["rz", "reference"])
    ap.add_argument("--config", default="scene_scale",
                    choices=["scene_scale", "random_triangles", "batch_views", "stress"])
    ap.add_argument("--views", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true", help="timed frames only (for ncu captures)")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-path comparison")
    ap.add_argument("--samples", type=int, default=1, choices=[1, 4],
                    help="camera-pass samples per pixel (4: the reference's 4x multisampling)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "rz":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "batch_views":
        run_batch(args)
    elif args.config == "stress":
        run_stress(args)
    else:
        run_rz(args)


if __name__ == "__main__":
    main()
