"""Benchmark of the hybrid pass: 1920x1080, 1.5M triangles, 4 area lights x 16
shadow samples (decorrelated RNG), mirror bounces, denoise accumulation on.

One step = one frame of the pass (shadow rays -> accumulation -> shading)
with the G-buffer already resident in HBM; the accumulation frame counter
advances every step as it does for a static camera in the reference.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  Under torchrun each rank renders its own frames
(replicas, no collective); value = rays of all ranks / max wall time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "hybrid_pass_mrays_per_s"
UNIT = "Mrays/s"
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU work of the baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--minb", type=int, default=0, help="shadow-kernel variant: resident blocks per SM")
    ap.add_argument("--workload", default="hd", choices=["hd", "batch"],
                    help="hd: the 1080p frame (headline); batch: 64 mixed views over 8 scenes, batched vs per view")
    ap.add_argument("--views", type=int, default=64)
    return ap.parse_args()


def workload(args):
    from vulkanhybridraytracer_gb300 import scenes

    return scenes.hd(1, args.width, args.height, spp=args.spp)


def config_of(wl, args):
    return {"workload": wl.name, "width": wl.width, "height": wl.height, "triangles": wl.scene.num_tris,
            "lights": len(wl.scene.lights), "shadow_spp": wl.spp, "rng": "decorrelated",
            "max_bounces": wl.max_bounces, "accumulation": "u8 history, running mean (frame > 0)",
            "gbuffer": "6 planes fp32 (88 B/px), primary-ray producer, untimed",
            "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MB write)"}


# ---- clocks sampling -------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- CPU baseline (the oracle restatement of the reference shaders) ---------------------
def cpu_run(wl, cam, planes_np, threads: int, target_s: float, frame: int):
    """Times the CPU restatement on a band of rows of the same frame, growing the
    band until it takes about target_s; returns (Mrays/s, sample description)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle as po

    po.set_threads(threads)
    orc = po.OracleScene()
    orc.set_scene(wl.scene)
    orc.build_bvh()
    H = planes_np[0].shape[0]
    rows = 4
    cfg = po.cfg_dict(spp=wl.spp, max_bounces=wl.max_bounces, rng_mode=wl.rng_mode, accum_frame=frame)
    while True:
        y0 = max(0, H // 2 - rows // 2)
        band = [np.ascontiguousarray(p[y0:y0 + rows]) for p in planes_np]
        hist = np.zeros((len(wl.scene.lights), rows, wl.width), np.uint8)
        t0 = time.perf_counter()
        _, _, _, st = orc.forward(band, cam, cfg, hist, 0)
        dt = time.perf_counter() - t0
        rays = st["shadow_rays"] + st["reflection_rays"] + st["hit_shadow_rays"]
        if dt >= target_s or rows >= H:
            break
        grow = max(2.0, min(8.0, target_s / max(dt, 1e-3)))
        rows = min(H, int(rows * grow))
    sample = (f"rows {y0}..{y0 + rows - 1} of the {wl.width}x{H} frame ({rows * wl.width} px, "
              f"{rays} rays), oracle forward pass, {threads} threads, {dt:.1f} s")
    return rays / dt / 1e6, sample, dt


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    """Reference arm: the reference's hybrid math on the host cores (its own
    Vulkan pipeline cannot run here), timed on bounded samples of the frame."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    wl = workload(args)
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle as po

    threads = os.cpu_count() or 1
    orc = po.OracleScene()
    orc.set_scene(wl.scene)
    orc.build_bvh()
    cam = wl.camera(1.0)
    planes = orc.gbuffer(cam, wl.width, wl.height)
    vals = []
    sample = ""
    per_step = max(1.0, args.cpu_seconds / 4)
    for i in range(args.warmup + args.steps):
        v, sample, _ = cpu_run(wl, cam, planes, threads, per_step, i + 1)
        if i >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals)) if vals else 0.0
    rays_per_frame = None
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_of(wl, args),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference Vulkan pipeline unavailable on this box (no graphics stack); the arm times the "
                    "CPU restatement of its shaders (oracle/) with all host threads"}
    del rays_per_frame
    print(json.dumps(line))


def run_batch(args):
    """64 views over 8 scenes (50k-2M triangles, 320x240..1920x1080, spp 1/4/16/64,
    1-8 lights): the views one by one through hy_hybrid_forward, then as one
    batch through hy_batch_forward (one persistent launch, CUDA-graph replay)."""
    import torch

    from vulkanhybridraytracer_gb300 import _lib as L
    from vulkanhybridraytracer_gb300 import autotune, scenes
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config

    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    scs, specs = scenes.batch(2, n_views=args.views)
    ctxs = []
    for sc in scs:
        c = HybridContext(0, stream=stream.cuda_stream)
        c.set_scene(sc)
        c.build_bvh()
        ctxs.append(c)
    runner = HybridContext(0, stream=stream.cuda_stream)
    views = []
    for sp in specs:
        sc = scs[sp["scene"]]
        w, h = sp["width"], sp["height"]
        cam = sp["camera"].rt_camera(w, h, 1.0)
        planes = ctxs[sp["scene"]].gbuffer(cam, w, h)
        hist = torch.zeros((sp["lights"], h, w), dtype=torch.uint8, device=dev)
        views.append(dict(scene=sp["scene"], planes=planes, camera=cam, hist=hist, spp=sp["spp"], sc=sc, w=w, h=h,
                          out_8=torch.empty((h, w, 4), dtype=torch.uint8, device=dev)))
    torch.cuda.synchronize()

    def set_frame(frame, chunk=1, minb=8):
        for v in views:
            v["camera"][32] = float(frame)
            v["config"] = pass_config(v["spp"], 1, L.HY_RNG_DECORRELATED, frame, L.HY_FLAG_NO_STATUS_SYNC,
                                      queue_chunk=chunk, min_blocks=minb)

    frame = [1]

    def plain():
        frame[0] += 1
        set_frame(frame[0])
        for v in views:
            ctxs[v["scene"]].forward(v["planes"], v["camera"], v["config"], v["hist"], out_8=v["out_8"], stats=False)

    def batched(chunk=1, minb=8):
        frame[0] += 1
        set_frame(frame[0])
        runner.batch_forward(ctxs, views, graph=True, tuning=pass_config(1, queue_chunk=chunk, min_blocks=minb),
                             sync=False)

    def dev_time(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3

    # rays per batch (counted once)
    set_frame(1)
    st = runner.batch_forward(ctxs, views, graph=False)
    rays = st["shadow_rays"] + st["reflection_rays"] + st["hit_shadow_rays"]
    sig = f"batch{len(views)}-{sum(v['w'] * v['h'] for v in views)}px-{rays}rays"
    tune = autotune.autotune(lambda ch, mb: batched(ch, mb), sig, torch.cuda.get_device_name(0), timer=dev_time)
    for _ in range(args.warmup):
        plain()
        batched(tune["chunk"], tune["min_blocks"])
    t_plain = [dev_time(plain) for _ in range(args.steps)]
    t_batch = [dev_time(lambda: batched(tune["chunk"], tune["min_blocks"])) for _ in range(args.steps)]
    mp = float(np.median(t_plain))
    mb = float(np.median(t_batch))
    line = {"metric": "hybrid_batch_mrays_per_s", "value": rays / mb / 1e6, "unit": "Mrays/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * mb, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"batch-{len(views)}views-8scenes", "views": len(views),
                       "scene_triangles": [c.num_tris for c in ctxs],
                       "pixels": sum(v["w"] * v["h"] for v in views), "rays_per_batch": rays,
                       "spp": [v["spp"] for v in views], "lights": [v["hist"].shape[0] for v in views],
                       "l2": "inputs (G-buffers ~%.1f GB) larger than L2" %
                             (sum(v["w"] * v["h"] for v in views) * 88 / 1e9)},
            "plain_per_view": {"value": rays / mp / 1e6, "unit": "Mrays/s", "ms_per_step": 1e3 * mp},
            "batched_over_plain": mp / mb,
            "autotune": tune,
            "gpu_launches": 2}
    print(json.dumps(line))
    for c in ctxs + [runner]:
        c.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from vulkanhybridraytracer_gb300 import _lib as L
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config

    wl = workload(args)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)  # torch ops and the library share one stream
    ctx = HybridContext(local, stream=stream.cuda_stream)
    ctx.set_scene(wl.scene)
    bvh = ctx.build_bvh()
    cam0 = wl.camera(1.0)
    planes = ctx.gbuffer(cam0, wl.width, wl.height)
    torch.cuda.synchronize()
    hist = ctx.new_history(wl.width, wl.height, L.HY_ACCUM_U8)
    out_f = torch.empty((wl.height, wl.width, 4), dtype=torch.float32, device=dev)
    out_8 = torch.empty((wl.height, wl.width, 4), dtype=torch.uint8, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def cfg(frame, flags=L.HY_FLAG_NO_STATUS_SYNC):
        return pass_config(spp=wl.spp, max_bounces=wl.max_bounces, rng_mode=wl.rng_mode, accum_frame=frame,
                           flags=flags, block_size=args.block, queue_chunk=args.chunk, min_blocks=args.minb)

    # rays per frame and traversal counts (untimed counting launch, same frame as step 1)
    st_count = ctx.forward(planes, wl.camera(1.0), cfg(1, L.HY_FLAG_COUNT_TRAVERSAL), hist.clone(),
                           L.HY_ACCUM_U8, out_f=out_f, out_8=out_8)
    st_plain = ctx.forward(planes, wl.camera(1.0), cfg(1, 0), hist.clone(), L.HY_ACCUM_U8, out_f=out_f,
                           out_8=out_8)
    rays = st_plain["shadow_rays"] + st_plain["reflection_rays"] + st_plain["hit_shadow_rays"]

    frame = 0
    for _ in range(args.warmup):
        frame += 1
        ctx.forward(planes, wl.camera(float(frame)), cfg(frame), hist, L.HY_ACCUM_U8, out_f=out_f, out_8=out_8)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    step_rays = []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    t_wall = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        frame += 1
        ev[k][0].record(stream)
        ctx.forward(planes, wl.camera(float(frame)), cfg(frame), hist, L.HY_ACCUM_U8, out_f=out_f, out_8=out_8)
        ev[k][1].record(stream)
        step_rays.append(rays)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = sum(ms) / 1e3
    if ws > 1:
        t = torch.tensor([t_dev], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_dev = float(t.item())
    total_rays = rays * args.steps * ws
    value = total_rays / t_dev / 1e6
    ms_per_step = t_dev * 1e3 / args.steps

    # roofline: algorithmic bytes per launch / launch time (the fused pass kernel)
    npx = wl.width * wl.height
    L_ = len(wl.scene.lights)
    alg_bytes = (rays * (32 + 16) + 80 * st_count["nodes_visited"] + 48 * st_count["tris_tested"]
                 + npx * (88 + 16 + 4 + 2 * L_))
    achieved = alg_bytes / (ms_per_step / 1e3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(ROOT / "MEASURED_PEAKS.json"))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = None
    tf = ROOT / "profiles" / "traffic_fused_hd.json"
    if tf.exists():
        try:
            traffic = json.load(open(tf)).get("bytes_per_launch")
        except Exception:
            traffic = None

    # e2e: host G-buffer in, host BGRA8 image out, through hy_hybrid_forward_host
    planes_h = [p.cpu().pin_memory() for p in planes]
    out8_h = torch.empty((wl.height, wl.width, 4), dtype=torch.uint8).pin_memory()
    h2d = sum(p.numel() * p.element_size() for p in planes_h)
    d2h = out8_h.numel()
    for _ in range(2):
        frame += 1
        ctx.forward_host(planes_h, wl.camera(float(frame)), cfg(frame, 0), hist, L.HY_ACCUM_U8, out_8=out8_h)
    e2e_t = []
    for _ in range(max(3, min(args.steps, 10))):
        frame += 1
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.forward_host(planes_h, wl.camera(float(frame)), cfg(frame, 0), hist, L.HY_ACCUM_U8, out_8=out8_h,
                         stats=False)
        e2e_t.append(time.perf_counter() - t0)
    e2e_value = rays / (sum(e2e_t) / len(e2e_t)) / 1e6 * ws

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        planes_np = [p.cpu().numpy() for p in planes]
        threads = os.cpu_count() or 1
        v, sample, _ = cpu_run(wl, wl.camera(1.0), planes_np, threads, args.cpu_seconds, 1)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_of(wl, args),
            "rays_per_frame": rays,
            "rays_breakdown": {k: st_plain[k] for k in ("shadow_rays", "reflection_rays", "hit_shadow_rays")},
            "traversal_per_ray": {"nodes": st_count["nodes_visited"] / rays, "tris": st_count["tris_tested"] / rays},
            "bvh": {"build_ms": bvh["build_ms"], "bvh8_nodes": bvh["num_bvh8_nodes"], "depth": bvh["depth"]},
            "wall_s": t_wall,
            "clocks": clk,
            "gpu_launches": 2 * args.steps,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * sum(e2e_t) / len(e2e_t)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_shadow (shadow rays + accumulation) and k_pixels<MODE_SHADE>, per frame",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"},
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
