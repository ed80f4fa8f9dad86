"""Benchmark of the hybrid pass: 1920x1080, 1.5M triangles, 4 area lights x 16
shadow samples (decorrelated RNG), mirror bounces, denoise accumulation on.

One step = one frame of the pass (shadow rays -> accumulation -> shading)
with the G-buffer already resident in HBM; the accumulation frame counter
advances every step as it does for a static camera in the reference.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  Under torchrun each rank renders its own frames
(replicas, no collective); value = rays of all ranks / max wall time.  On
rank 0 the line also carries the two other legs of the headline metric:
"batch" (64 mixed views over 8 scenes, batched against view by view) and
"diff" (512x512 forward + adjoint, backward / forward time, gradient check
against central differences).
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
    ap.add_argument("--group", type=int, default=0, help="lanes per pixel-light group (0: next power of 2 >= spp)")
    ap.add_argument("--visits", type=int, default=0, help="node visits per scheduling round of the shadow kernel")
    ap.add_argument("--sched", default="stream", choices=["stream", "groups", "pool"],
                    help="DECORRELATED shadow samples: tile streams, fixed lane groups or the per-warp ray pool")
    ap.add_argument("--workload", default="hd", choices=["hd", "batch", "diff", "pathtrace", "large"],
                    help="hd: the 1080p frame (headline); batch: 64 mixed views over 8 scenes, batched vs per "
                         "view; diff: 512x512 forward + adjoint; pathtrace: the path-traced mode at 1080p; "
                         "large: 4K, 7.35M triangles, 64 lights, forward + adjoint + batch")
    ap.add_argument("--views", type=int, default=64)
    ap.add_argument("--no-legs", action="store_true", help="skip the batch and diff legs of the default line")
    ap.add_argument("--mirror-reflection", action="store_true",
                    help="the reference's perfect mirror reflection instead of the configuration's GGX-sampled ray")
    ap.add_argument("--leg-steps", type=int, default=3, help="timed steps of the batch and diff legs")
    ap.add_argument("--large-div", type=int, default=1,
                    help="large workload: the 4K resolution divided by this (small ncu cases); the scene is unchanged")
    ap.add_argument("--anyhit", default="auto", choices=["auto", "far", "near"],
                    help="any-hit child order of the scenes (hy_scene_set_anyhit_order)")
    ap.add_argument("--no-tune", action="store_true",
                    help="batch workload: the default launch shape instead of the autotuner's sweep")
    ap.add_argument("--build-mode", default="sah", choices=["sah", "lbvh"],
                    help="binary tree under the 8-wide nodes (hy_scene_set_build_mode)")
    return ap.parse_args()


def workload(args):
    from vulkanhybridraytracer_gb300 import scenes

    return scenes.hd(1, args.width, args.height, spp=args.spp)


ANYHIT_ORDER = {1: "far first", 2: "near first"}  # HY_ANYHIT_FAR_FIRST / HY_ANYHIT_NEAR_FIRST

# device sources of the pass kernels: a profile summary under profiles/ records the hash
# of these files, so a figure measured on another version of the kernels is not reported
# as this version's
KERNEL_SOURCES = ("hy_device.cuh", "hy_stream.cuh", "hy_stream_kernel.cuh", "hy_stream_accum.cu", "hy_shade.cuh",
                  "hy_pass.h", "hy_pass.cu", "hy_bvh.cu", "hy_sah.cu")


def code_of(text: str) -> str:
    """C++/CUDA source without comments and blank lines (what the hash covers)."""
    import re

    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    lines = (re.sub(r"//.*$", "", ln).rstrip() for ln in text.splitlines())
    return "\n".join(ln for ln in lines if ln.strip())


def kernel_source_sha(read=None) -> str:
    """Hash of the code (comments stripped) of the kernels and structure build."""
    import hashlib

    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        text = read(f) if read else (ROOT / "vulkanhybridraytracer_gb300" / "csrc" / f).read_text()
        h.update(code_of(text).encode())
    return h.hexdigest()[:16]


def profile_records(kernel: str) -> dict:
    """`bench_record <kernel> key=value ...` lines of the ncu summaries in profiles/:
    {key: (value, file)} for this kernel."""
    out = {}
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for ln in f.read_text().splitlines():
            parts = ln.split()
            if len(parts) >= 3 and parts[0] == "bench_record" and parts[1] == kernel:
                for kv in parts[2:]:
                    k, _, v = kv.partition("=")
                    out[k] = (v, f"profiles/{f.name}")
    return out


# the 1080p configuration's reflection ray: GGX-sampled for roughness < 0.3 texels
# (shading model 3 in the synthetic scenes); --mirror-reflection keeps the reference's
# perfect reflect()
def reflection_flags(args) -> int:
    from vulkanhybridraytracer_gb300 import _lib as L

    return 0 if args.mirror_reflection else L.HY_FLAG_GGX_REFLECTION


def config_of(wl, args):
    return {"workload": wl.name, "width": wl.width, "height": wl.height, "triangles": wl.scene.num_tris,
            "lights": len(wl.scene.lights), "shadow_spp": wl.spp, "rng": "decorrelated",
            "reflection": ("perfect mirror (reflect)" if args.mirror_reflection else
                           "GGX-sampled from the texel's lobe (roughness < 0.3 texels), 1 ray"),
            "max_bounces": wl.max_bounces, "accumulation": "u8 history, running mean (frame > 0)",
            "gbuffer": "6 planes fp32 (88 B/px), primary-ray producer, untimed",
            "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MB write)",
            "structure": STRUCTURE[BUILD_MODE["mode"]]}


BUILD_MODE = {"mode": "sah", "anyhit": "auto"}
STRUCTURE = {"sah": "binned SAH (32 bins per axis) binary tree -> compressed BVH8",
             "lbvh": "LBVH (Karras radix tree over 30-bit Morton codes) -> compressed BVH8"}


def build_structure(ctx, instanced: bool = False):
    """hy_bvh_build(_instanced) with the build mode of --build-mode and the any-hit order of --anyhit."""
    from vulkanhybridraytracer_gb300 import _lib as L

    ctx.set_build_mode(L.HY_BUILD_SAH if BUILD_MODE["mode"] == "sah" else L.HY_BUILD_LBVH)
    ctx.set_anyhit_order({"auto": L.HY_ANYHIT_AUTO, "far": L.HY_ANYHIT_FAR_FIRST,
                          "near": L.HY_ANYHIT_NEAR_FIRST}[BUILD_MODE["anyhit"]])
    return ctx.build_bvh(instanced=instanced)


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
def cpu_run(wl, cam, planes_np, threads: int, target_s: float, frame: int, flags: int = 0):
    """Times the CPU restatement on a band of rows of the same frame, growing the
    band until it takes about target_s; returns (Mrays/s, sample description)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle as po

    po.set_threads(threads)
    orc = po.OracleScene()
    orc.set_scene(wl.scene)
    orc.set_build_mode(po.HY_BUILD_SAH if BUILD_MODE["mode"] == "sah" else po.HY_BUILD_LBVH)
    orc.build_bvh()
    H = planes_np[0].shape[0]
    rows = 4
    cfg = po.cfg_dict(spp=wl.spp, max_bounces=wl.max_bounces, rng_mode=wl.rng_mode, accum_frame=frame, flags=flags)
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
    orc.set_build_mode(po.HY_BUILD_SAH if BUILD_MODE["mode"] == "sah" else po.HY_BUILD_LBVH)
    orc.build_bvh()
    cam = wl.camera(1.0)
    planes = orc.gbuffer(cam, wl.width, wl.height)
    vals = []
    sample = ""
    per_step = max(1.0, args.cpu_seconds / 4)
    for i in range(args.warmup + args.steps):
        v, sample, _ = cpu_run(wl, cam, planes, threads, per_step, i + 1, reflection_flags(args))
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


def diff_leg(steps: int, warmup: int, fd_params: int = 32, clocks_index: int = 0, visits: int = 0) -> dict:
    """Differentiable form: 512x512, 64 icospheres (subdivision 3), 64 materials, 8 point
    lights, 16 shadow samples; L2 loss against a target rendered from parameters perturbed
    by N(0, 0.05).  Forward = G-buffer + shadow pass + shading at the current parameters;
    backward = hy_hybrid_backward (visibility held fixed).  The gradient is checked against
    central differences of the same FP32 forward on `fd_params` seeded parameters, with
    the shadow images held fixed (the adjoint's visibility) and the loss summed in FP64."""
    import torch

    from vulkanhybridraytracer_gb300 import diffrender, scenes

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    wl = scenes.diff(3, 512, 512)
    r = diffrender.DiffRenderer(wl.scene, wl.camera(0.0), wl.width, wl.height, spp=wl.spp,
                                max_bounces=wl.max_bounces)
    if visits:  # node visits per scheduling round of the shadow kernel (--visits)
        from vulkanhybridraytracer_gb300.hybrid import pass_config
        r.cfg = pass_config(spp=wl.spp, max_bounces=wl.max_bounces, rng_mode=r.cfg.rng_mode, visits_per_round=visits)
    mp0, lp0 = r.params0
    rng = np.random.default_rng(3)
    mp_t = np.clip(mp0 + rng.normal(0, 0.05, mp0.shape), 0.0, 1.0).astype(np.float32)
    lp_t = (lp0 + rng.normal(0, 0.05, lp0.shape)).astype(np.float32)
    target, _ = r.render(mp_t, lp_t)
    target = target.clone()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step():
        r.set_params(mp0, lp0)
        flush.zero_()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record(stream)
        planes = r.ctx.gbuffer(r.cam, r.W, r.H)
        shadow = torch.zeros((r.ctx.num_lights, r.H, r.W), dtype=torch.float32, device=dev)
        r.ctx.shadow_pass(planes, r.cam, r.cfg, shadow, r.fmt)
        img = torch.empty((r.H, r.W, 4), dtype=torch.float32, device=dev)
        r.ctx.shade_pass(planes, r.cam, r.cfg, shadow, r.fmt, out_f=img)
        e[1].record(stream)
        grad = 2.0 * (img - target)
        grad[..., 3] = 0.0
        e[2].record(stream)
        gm, gl, st = r.backward((planes, shadow), grad)
        e[3].record(stream)
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3]), st, (planes, shadow, img, gm, gl)

    for _ in range(warmup):
        step()
    fw, bw = [], []
    clocks = Clocks(clocks_index)
    clocks.start()
    for _ in range(steps):
        f, b, st, state = step()
        fw.append(f)
        bw.append(b)
    clk = clocks.stop()
    planes, shadow, img, gm, gl = state
    loss0 = float(((img - target)[..., :3].double() ** 2).sum())

    # central differences of the FP32 forward, visibility (shadow images) held fixed
    g = np.concatenate([gm.cpu().numpy().ravel(), gl.cpu().numpy().ravel()]).astype(np.float64)
    p0 = np.concatenate([mp0.ravel(), lp0.ravel()]).astype(np.float64)
    nm = mp0.size
    scale = float(np.abs(g).max())
    cand = np.flatnonzero(np.abs(g) > 1e-2 * scale)
    pick = np.random.default_rng(1).choice(cand, size=min(fd_params, len(cand)), replace=False)
    out = torch.empty((r.H, r.W, 4), dtype=torch.float32, device=dev)

    def loss(p):
        r.set_params(p[:nm].reshape(mp0.shape).astype(np.float32), p[nm:].reshape(lp0.shape).astype(np.float32))
        pl = r.ctx.gbuffer(r.cam, r.W, r.H)
        r.ctx.shade_pass(pl, r.cam, r.cfg, shadow, r.fmt, out_f=out)
        return float(((out - target)[..., :3].double() ** 2).sum())

    fd = []
    for j in pick:
        # small steps: a light moved by h also moves the shadow rays the shading traces
        # from bounce hits, whose visibility the adjoint holds fixed
        h = 1e-3 * max(1.0, abs(p0[j]))
        a, b = p0.copy(), p0.copy()
        a[j] += h
        b[j] -= h
        fd.append((loss(a) - loss(b)) / (2 * h))
    fd = np.array(fd)
    rel = np.abs(g[pick] - fd) / np.maximum(np.abs(fd), 1e-2 * scale)
    r.set_params(mp0, lp0)
    f_ms, b_ms = float(np.mean(fw)), float(np.mean(bw))
    out = {"workload": wl.name, "width": wl.width, "height": wl.height, "triangles": wl.scene.num_tris,
           "materials": len(wl.scene.materials), "lights": len(wl.scene.lights), "shadow_spp": wl.spp,
           "max_bounces": wl.max_bounces, "params": len(wl.scene.materials) * 5 + len(wl.scene.lights) * 4,
           "loss": loss0, "loss_kind": "L2 vs target rendered from params + N(0, 0.05)",
           "forward_ms": f_ms, "backward_ms": b_ms, "backward_over_forward": b_ms / f_ms,
           "forward_parts": "G-buffer + 16-spp shadow pass + shading",
           "backward_rays": {"reflection_rays": st["reflection_rays"], "hit_shadow_rays": st["hit_shadow_rays"]},
           "grad_check": {"params": int(len(pick)), "max_rel_err": float(rel.max()) if len(rel) else None,
                          "median_rel_err": float(np.median(rel)) if len(rel) else None,
                          "max_rel_err_materials": float(rel[pick < nm].max()) if np.any(pick < nm) else None,
                          "max_rel_err_lights": float(rel[pick >= nm].max()) if np.any(pick >= nm) else None,
                          "method": "central differences of the FP32 forward (h = 1e-3 max(1, |p|)), shadow "
                                    "images held fixed, loss summed in FP64; relative to max(|fd|, 1e-2 max|grad|)"},
           "steps": steps, "warmup": warmup, "clocks": clk,
           "l2": f"flushed between steps ({L2_FLUSH_BYTES >> 20} MB write)"}
    r.close()
    return out


def run_diff(args):
    import torch

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream(device=torch.device("cuda", 0))
    torch.cuda.set_stream(stream)
    d = diff_leg(args.steps, args.warmup, visits=args.visits)
    line = {"metric": "hybrid_backward_ms", "value": d["backward_ms"], "unit": "ms", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": d["backward_ms"], "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {k: d[k] for k in ("workload", "width", "height", "triangles", "materials", "lights",
                                         "shadow_spp", "max_bounces", "params", "loss_kind", "l2")},
            "forward_ms": d["forward_ms"], "backward_over_forward": d["backward_over_forward"],
            "backward_rays": d["backward_rays"], "grad_check": d["grad_check"], "loss": d["loss"],
            "clocks": d["clocks"], "gpu_launches": 2}
    print(json.dumps(line))


def run_pathtrace(args):
    """Path-traced mode on the 1080p / 1.5M-triangle scene: camera rays, up to 8 mirror/glass
    segments, args.spp decorrelated shadow rays per light at every hit, running mean into
    the BGRA8 image."""
    import torch

    from vulkanhybridraytracer_gb300 import _lib as L
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    wl = workload(args)
    ctx = HybridContext(0, stream=stream.cuda_stream)
    ctx.set_scene(wl.scene)
    build_structure(ctx)
    img = torch.zeros((wl.height, wl.width, 4), dtype=torch.uint8, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    cfg = pass_config(spp=wl.spp, max_bounces=8, rng_mode=L.HY_RNG_DECORRELATED, flags=L.HY_FLAG_NO_STATUS_SYNC,
                      min_blocks=args.minb, visits_per_round=args.visits)
    _, st = ctx.pathtrace(wl.camera(0.0), wl.width, wl.height, pass_config(wl.spp, 8, L.HY_RNG_DECORRELATED), img)
    rays = st["shadow_rays"] + st["reflection_rays"]
    for f in range(args.warmup):
        ctx.pathtrace(wl.camera(float(f + 1)), wl.width, wl.height, cfg, img, stats=False)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = Clocks(0)
    ctx.profile(True)
    clocks.start()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        ctx.pathtrace(wl.camera(float(args.warmup + k + 1)), wl.width, wl.height, cfg, img, stats=False)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    kernels = ctx.profile_read()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    line = {"metric": "pathtrace_mrays_per_s", "value": rays / (ms / 1e3) / 1e6, "unit": "Mrays/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": wl.name.replace("hd-", "pathtrace-"), "width": wl.width, "height": wl.height,
                       "triangles": wl.scene.num_tris, "lights": len(wl.scene.lights), "shadow_spp": wl.spp,
                       "rng": "decorrelated", "max_bounces": 8,
                       "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MB write)",
            "structure": STRUCTURE[BUILD_MODE["mode"]]},
            "rays_per_frame": rays, "rays_breakdown": {"shadow_rays": st["shadow_rays"],
                                                       "camera_and_bounce_rays": st["reflection_rays"]},
            "per_kernel": kernels, "clocks": clk, "gpu_launches": args.steps}
    print(json.dumps(line))
    ctx.close()


def run_large(args):
    """The large combined configuration: 3840x2160, 4096 instances of 8 base meshes + the
    terrain (8.81M triangles in one BVH8), 64 area lights x 1 sample, 2 bounces; the frame,
    its adjoint over 1024 materials and 64 lights, and the frame batched with 4 extra 1080p
    views (hy_batch_forward) against the same 5 views one by one."""
    import torch

    from vulkanhybridraytracer_gb300 import _lib as L
    from vulkanhybridraytracer_gb300 import scenes
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config
    from vulkanhybridraytracer_gb300.scene import Camera

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    wl = scenes.large(width=3840 // args.large_div, height=2160 // args.large_div)
    ctx = HybridContext(0, stream=stream.cuda_stream)
    ctx.set_scene(wl.scene)
    bvh = build_structure(ctx)
    W, H, NL = wl.width, wl.height, len(wl.scene.lights)
    cam0 = wl.camera(1.0)
    planes = ctx.gbuffer(cam0, W, H)
    hist = torch.zeros((NL, H, W), dtype=torch.uint8, device=dev)
    out8 = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
    outf = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def cfg(frame, flags=L.HY_FLAG_NO_STATUS_SYNC):
        return pass_config(spp=1, max_bounces=wl.max_bounces, rng_mode=L.HY_RNG_DECORRELATED, accum_frame=frame,
                           flags=flags, min_blocks=args.minb, visits_per_round=args.visits)

    st = ctx.forward(planes, wl.camera(0.0), cfg(0, 0), hist, L.HY_ACCUM_U8, out_f=outf, out_8=out8)
    rays = st["shadow_rays"] + st["reflection_rays"] + st["hit_shadow_rays"]
    frame = 0
    for _ in range(args.warmup):
        frame += 1
        ctx.forward(planes, wl.camera(float(frame)), cfg(frame), hist, L.HY_ACCUM_U8, out_f=outf, out_8=out8)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    fw = []
    for _ in range(args.steps):
        flush.zero_()
        frame += 1
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.forward(planes, wl.camera(float(frame)), cfg(frame), hist, L.HY_ACCUM_U8, out_f=outf, out_8=out8)
        b.record(stream)
        fw.append((a, b))
    torch.cuda.synchronize()
    f_ms = float(np.mean([a.elapsed_time(b) for a, b in fw]))

    # adjoint of the frame's shading (dLoss/dImage: a fixed random image)
    g = torch.randn((H, W, 4), generator=torch.Generator(device=dev).manual_seed(4), device=dev)
    g[..., 3] = 0
    bw = []
    bcfg = cfg(frame, 0)
    for k in range(args.warmup + args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        gm, gl, bst = ctx.backward(planes, wl.camera(float(frame)), bcfg, hist, g, L.HY_ACCUM_U8)
        b.record(stream)
        if k >= args.warmup:
            bw.append((a, b))
    torch.cuda.synchronize()
    b_ms = float(np.mean([a.elapsed_time(b) for a, b in bw]))

    # the frame batched with 4 extra 1080p views of the same scene
    views = [dict(planes=planes, w=W, h=H, hist=hist, out_8=out8, cam=lambda f: wl.camera(f))]
    for i in range(4):
        ang = 2 * np.pi * (i + 0.5) / 4
        c = Camera((50.0 * np.sin(ang), 20.0, 50.0 * np.cos(ang)), (0.0, 0.0, 0.0), 60.0)
        p = ctx.gbuffer(c.rt_camera(1920, 1080, 1.0), 1920, 1080)
        views.append(dict(planes=p, w=1920, h=1080, out_8=torch.empty((1080, 1920, 4), dtype=torch.uint8, device=dev),
                          hist=torch.zeros((NL, 1080, 1920), dtype=torch.uint8, device=dev),
                          cam=lambda f, c=c: c.rt_camera(1920, 1080, f)))
    torch.cuda.synchronize()

    def batch_views(f):
        return [dict(scene=0, planes=v["planes"], camera=v["cam"](float(f)), config=cfg(f), hist=v["hist"],
                     out_8=v["out_8"]) for v in views]

    def time_it(fn, reps):
        ts = []
        for _ in range(reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            ts.append((a, b))
        torch.cuda.synchronize()
        return float(np.mean([a.elapsed_time(b) for a, b in ts]))

    bf = [frame]

    def plain():
        bf[0] += 1
        for v in batch_views(bf[0]):
            ctx.forward(v["planes"], v["camera"], v["config"], v["hist"], L.HY_ACCUM_U8, out_8=v["out_8"],
                        stats=False)

    def batched():
        bf[0] += 1
        ctx.batch_forward([ctx], batch_views(bf[0]), graph=True, sync=False)

    for _ in range(2):
        plain()
        batched()
    st_b = ctx.batch_forward([ctx], batch_views(bf[0] + 1), graph=True, sync=True)
    bf[0] += 1
    rays_b = st_b["shadow_rays"] + st_b["reflection_rays"] + st_b["hit_shadow_rays"]
    mp = time_it(plain, args.steps)
    mb = time_it(batched, args.steps)

    # the same frame over the two-level structure (8 mesh BLASes + the terrain's
    # under a TLAS of 4097 instances), and the per-frame structure update of both
    xf = wl.scene.pack()[3]
    ctx2 = HybridContext(0, stream=stream.cuda_stream)
    ctx2.set_scene(wl.scene)
    bvh2 = build_structure(ctx2, instanced=True)
    order2 = ANYHIT_ORDER[ctx2.anyhit_order()]
    lay2 = ctx2.bvh_layout()
    st2 = ctx2.forward(planes, wl.camera(0.0), cfg(0, 0), hist, L.HY_ACCUM_U8, out_f=outf, out_8=out8)
    rays2 = st2["shadow_rays"] + st2["reflection_rays"] + st2["hit_shadow_rays"]
    f2 = [frame]

    def fwd2():
        f2[0] += 1
        ctx2.forward(planes, wl.camera(float(f2[0])), cfg(f2[0]), hist, L.HY_ACCUM_U8, out_f=outf, out_8=out8,
                     stats=False)

    for _ in range(args.warmup):
        fwd2()
    f2_ms = time_it(fwd2, args.steps)

    def update_ms(c):
        ts = []
        for _ in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            c.refit_bvh(xf)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return 1e3 * float(np.median(ts[args.warmup:]))

    upd_flat, upd_two = update_ms(ctx), update_ms(ctx2)
    ctx2.close()
    clk = clocks.stop()
    line = {"metric": "large_combined_mrays_per_s", "value": rays / (f_ms / 1e3) / 1e6, "unit": "Mrays/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": f_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": wl.name, "width": W, "height": H, "triangles": wl.scene.num_tris,
                       "instances": len(wl.scene.entities) - 1, "materials": len(wl.scene.materials),
                       "lights": NL, "shadow_spp_per_light": 1, "max_bounces": wl.max_bounces,
                       "rng": "decorrelated", "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MB write)"},
            "bvh": {"build_ms": bvh["build_ms"], "bvh8_nodes": bvh["num_bvh8_nodes"], "depth": bvh["depth"],
                    "anyhit_order": ANYHIT_ORDER[ctx.anyhit_order()]},
            "rays_per_frame": rays,
            "adjoint": {"backward_ms": b_ms, "backward_over_forward": b_ms / f_ms,
                        "params": len(wl.scene.materials) * 5 + NL * 4,
                        "rays_retraced": bst["reflection_rays"] + bst["hit_shadow_rays"]},
            "batch_4k_plus_4x1080p": {"rays": rays_b, "batched_ms": mb, "per_view_ms": mp,
                                      "batched_mrays_per_s": rays_b / (mb / 1e3) / 1e6,
                                      "batched_over_per_view": mp / mb},
            "two_level": {"build_ms": bvh2["build_ms"], "nodes": lay2["num_nodes"], "blas": lay2["num_blas"],
                          "anyhit_order": order2,
                          "instances": lay2["num_instances"], "depth": lay2["depth"],
                          "node_bytes": lay2["num_nodes"] * 80, "flat_node_bytes": bvh["num_bvh8_nodes"] * 80,
                          "rays": rays2, "forward_ms": f2_ms, "mrays_per_s": rays2 / (f2_ms / 1e3) / 1e6,
                          "update_ms": upd_two, "flat_refit_ms": upd_flat},
            "clocks": clk, "gpu_launches": 2}
    print(json.dumps(line))
    ctx.close()


def batch_leg(steps: int, warmup: int, n_views: int = 64, tune: bool = False, clocks_index: int = 0) -> dict:
    """64 views over 8 scenes (50k-2M triangles, 320x240..1920x1080, spp 1/4/16/64,
    1-8 lights): the views one by one through hy_hybrid_forward, then as one
    batch through hy_batch_forward (one persistent launch, CUDA-graph replay).
    tune: sweep the launch shapes (autotune) instead of the defaults / the cache."""
    import torch

    from vulkanhybridraytracer_gb300 import _lib as L
    from vulkanhybridraytracer_gb300 import autotune, scenes
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    scs, specs = scenes.batch(2, n_views=n_views)
    ctxs = []
    for sc in scs:
        c = HybridContext(0, stream=stream.cuda_stream)
        c.set_scene(sc)
        build_structure(c)
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

    def set_frame(frame, chunk=1, minb=0):
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

    def batched(shape=autotune.DEFAULT):
        frame[0] += 1
        set_frame(frame[0])
        runner.batch_forward(ctxs, views, graph=True, tuning=autotune.tuning_config(shape), sync=False)

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
    if tune:
        frame[0] += 1
        set_frame(frame[0])
        tuned = autotune.autotune(runner, ctxs, views, sig, torch.cuda.get_device_name(0))
    else:
        tuned = autotune.cached(sig, torch.cuda.get_device_name(0)) or dict(autotune.DEFAULT, cached=False,
                                                                            default=True)
    for _ in range(warmup):
        plain()
        batched(tuned)
    clocks = Clocks(clocks_index)
    clocks.start()
    t_plain = [dev_time(plain) for _ in range(steps)]
    t_batch = [dev_time(lambda: batched(tuned)) for _ in range(steps)]
    clk = clocks.stop()
    mp = float(np.median(t_plain))
    mb = float(np.median(t_batch))
    # per-view census for the launch-list analysis of the view-by-view path: one
    # more view-by-view pass with its rays counted (the launches of this pass are
    # the last 64 shadow + shade pairs of the run)
    frame[0] += 1
    set_frame(frame[0])
    view_rays = []
    for v in views:
        sv = ctxs[v["scene"]].forward(v["planes"], v["camera"], v["config"], v["hist"], out_8=v["out_8"])
        view_rays.append(int(sv["shadow_rays"] + sv["reflection_rays"] + sv["hit_shadow_rays"]))
    out = {"workload": f"batch-{len(views)}views-8scenes", "views": len(views),
           "scene_triangles": [c.num_tris for c in ctxs],
           "pixels": sum(v["w"] * v["h"] for v in views), "rays_per_batch": rays,
           "spp": [v["spp"] for v in views], "lights": [v["hist"].shape[0] for v in views],
           "view_res": [f"{v['w']}x{v['h']}" for v in views], "view_rays": view_rays,
           "batched_ms": 1e3 * mb, "plain_ms": 1e3 * mp, "batched_over_plain": mp / mb,
           "batched_mrays_per_s": rays / mb / 1e6, "plain_mrays_per_s": rays / mp / 1e6,
           "tuning": {k: tuned[k] for k in ("chunk", "block", "min_blocks", "stack_depth", "cached") if k in tuned},
           "steps": steps, "warmup": warmup, "clocks": clk,
           "l2": "inputs (G-buffers ~%.1f GB) larger than L2" % (sum(v["w"] * v["h"] for v in views) * 88 / 1e9)}
    if tune:
        out["autotune"] = tuned
    for c in ctxs + [runner]:
        c.close()
    return out


def run_batch(args):
    import torch

    stream = torch.cuda.Stream(device=torch.device("cuda", 0))
    torch.cuda.set_stream(stream)
    d = batch_leg(args.steps, args.warmup, args.views, tune=not args.no_tune)
    line = {"metric": "hybrid_batch_mrays_per_s", "value": d["batched_mrays_per_s"], "unit": "Mrays/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": d["batched_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {k: d[k] for k in ("workload", "views", "scene_triangles", "pixels", "rays_per_batch", "spp",
                                         "lights", "l2")},
            "plain_per_view": {"value": d["plain_mrays_per_s"], "unit": "Mrays/s", "ms_per_step": d["plain_ms"]},
            "batched_over_plain": d["batched_over_plain"], "autotune": d.get("autotune"), "clocks": d["clocks"],
            "view_res": d["view_res"], "view_rays": d["view_rays"], "gpu_launches": 2}
    print(json.dumps(line))


def main():
    args = parse()
    BUILD_MODE["mode"] = args.build_mode
    BUILD_MODE["anyhit"] = args.anyhit
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "diff":
        run_diff(args)
        return
    if args.workload == "pathtrace":
        run_pathtrace(args)
        return
    if args.workload == "large":
        run_large(args)
        return
    import torch

    from vulkanhybridraytracer_gb300 import replicas

    ws, rank, local = replicas.env()
    torch.cuda.set_device(local)
    replicas.init()  # replicas: each rank renders its own frames, no data-path collective
    dev = torch.device("cuda", local)
    from vulkanhybridraytracer_gb300 import _lib as L
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config

    wl = workload(args)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)  # torch ops and the library share one stream
    ctx = HybridContext(local, stream=stream.cuda_stream)
    ctx.set_scene(wl.scene)
    bvh = build_structure(ctx)
    cam0 = wl.camera(1.0)
    planes = ctx.gbuffer(cam0, wl.width, wl.height)
    torch.cuda.synchronize()
    hist = ctx.new_history(wl.width, wl.height, L.HY_ACCUM_U8)
    out_f = torch.empty((wl.height, wl.width, 4), dtype=torch.float32, device=dev)
    out_8 = torch.empty((wl.height, wl.width, 4), dtype=torch.uint8, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    sched = {"pool": L.HY_FLAG_RAY_POOL, "groups": L.HY_FLAG_LANE_GROUPS}.get(args.sched, 0) | reflection_flags(args)

    def cfg(frame, flags=L.HY_FLAG_NO_STATUS_SYNC):
        return pass_config(spp=wl.spp, max_bounces=wl.max_bounces, rng_mode=wl.rng_mode, accum_frame=frame,
                           flags=flags | sched, block_size=args.block, queue_chunk=args.chunk, min_blocks=args.minb,
                           group_lanes=args.group, visits_per_round=args.visits)

    # rays per frame and traversal counts (untimed counting launch, same frame as step 1)
    st_count = ctx.forward(planes, wl.camera(1.0), cfg(1, L.HY_FLAG_COUNT_TRAVERSAL), hist.clone(),
                           L.HY_ACCUM_U8, out_f=out_f, out_8=out_8)
    st_plain = ctx.forward(planes, wl.camera(1.0), cfg(1, 0), hist.clone(), L.HY_ACCUM_U8, out_f=out_f,
                           out_8=out_8)
    rays = st_plain["shadow_rays"] + st_plain["reflection_rays"] + st_plain["hit_shadow_rays"]
    # the shadow kernel's own traversal counts (same rays as the fused frame)
    shadow_tmp = torch.empty((len(wl.scene.lights), wl.height, wl.width), dtype=torch.uint8, device=dev)
    st_shadow = ctx.shadow_pass(planes, wl.camera(1.0), cfg(1, L.HY_FLAG_COUNT_TRAVERSAL), shadow_tmp,
                                L.HY_ACCUM_U8)
    del shadow_tmp

    frame = 0
    for _ in range(args.warmup):
        frame += 1
        ctx.forward(planes, wl.camera(float(frame)), cfg(frame), hist, L.HY_ACCUM_U8, out_f=out_f, out_8=out_8)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    step_rays = []
    replicas.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    ctx.profile(True)  # CUDA events around each kernel launch, on the library's (= torch's) stream
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
    kernels = ctx.profile_read()
    ctx.profile(False)
    ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = replicas.max_over_ranks(sum(ms) / 1e3, dev)
    value = replicas.throughput(rays * args.steps, t_dev, ws) / 1e6
    ms_per_step = t_dev * 1e3 / args.steps

    # roofline of each kernel: algorithmic bytes per launch (48 B per ray record, 80 B per BVH8 node
    # visited, 48 B per triangle tested, plus the compulsory pixel I/O) / its average launch time
    npx = wl.width * wl.height
    L_ = len(wl.scene.lights)
    sh_rays = st_shadow["shadow_rays"]
    sh_nodes, sh_tris = st_shadow["nodes_visited"], st_shadow["tris_tested"]
    shadow_bytes = sh_rays * 48 + 80 * sh_nodes + 48 * sh_tris + npx * (32 + 2 * L_)
    alg = {
        # G-buffer planes 0/1 (32 B/px), u8 history read + write per light
        "k_shadow_stream<accum>": shadow_bytes,
        "k_shadow_group<accum>": shadow_bytes,
        "k_shadow_pool<accum>": shadow_bytes,
        # all six planes (88 B/px), RGBA32F + BGRA8 out, u8 history read per light
        "k_pixels<shade>": ((rays - sh_rays) * 48 + 80 * (st_count["nodes_visited"] - sh_nodes)
                            + 48 * (st_count["tris_tested"] - sh_tris) + npx * (88 + 16 + 4 + L_)),
    }
    alg_frame = shadow_bytes + alg["k_pixels<shade>"]
    peaks = {}
    try:
        peaks = json.load(open(ROOT / "MEASURED_PEAKS.json"))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    per_kernel = {}
    for name, k in kernels.items():
        e = {"launches": k["launches"], "avg_ms": k["avg_ms"],
             "share": k["total_ms"] / max(sum(x["total_ms"] for x in kernels.values()), 1e-9)}
        if name in alg:
            e["alg_bytes"] = alg[name]
            e["achieved_gbs"] = alg[name] / (k["avg_ms"] / 1e3) / 1e9
        per_kernel[name] = e
    dom = max(kernels, key=lambda n: kernels[n]["total_ms"]) if kernels else None
    if dom in alg:
        achieved = per_kernel[dom]["achieved_gbs"]
    else:  # no per-kernel record: the whole frame
        dom = "frame"
        achieved = alg_frame / (ms_per_step / 1e3) / 1e9
    # DRAM bytes per launch and the issue counters from the committed ncu summaries
    # (profiles/), used only when they were measured on these kernel sources
    rec = profile_records(dom)
    cur_sha = kernel_source_sha()

    def rec_val(key, conv=float):
        v = rec.get(key)
        if v is None or rec.get("source_sha", ("", ""))[0] != cur_sha:
            return None
        return conv(v[0])

    wkey = f"{wl.width}x{wl.height}"
    traffic = rec_val(f"dram_bytes_{wkey}", int)
    evidence = {"source_sha": cur_sha, "profile_sha": rec.get("source_sha", (None,))[0],
                "current": rec.get("source_sha", ("",))[0] == cur_sha,
                "files": sorted({v[1] for v in rec.values()}),
                "issue_active_pct": rec_val("issue_active_pct"),
                "lanes_per_inst": rec_val("lanes_per_inst"),
                "alu_pipe_pct": rec_val("alu_pipe_pct"),
                "l2_gbs": rec_val("l2_gbs"), "l2_bytes_per_launch": rec_val("l2_bytes"),
                "dram_gbs": rec_val("dram_gbs"), "profiled_case": rec.get("case", (None,))[0]}

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
        v, sample, _ = cpu_run(wl, wl.camera(1.0), planes_np, threads, args.cpu_seconds, 1, reflection_flags(args))
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
            "bvh": {"build_ms": bvh["build_ms"], "bvh8_nodes": bvh["num_bvh8_nodes"], "depth": bvh["depth"],
                    "anyhit_order": ANYHIT_ORDER[ctx.anyhit_order()]},
            "wall_s": t_wall,
            "clocks": clk,
            "gpu_launches": 2 * args.steps,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * sum(e2e_t) / len(e2e_t)},
            # the dominant kernel's algorithmic bytes against the measured HBM copy
            # bandwidth; what bounds it is instruction issue (ncu: issue-active
            # share, active lanes per instruction, ALU pipe), not DRAM, whose traffic
            # is a fraction of a percent of the algorithmic bytes (the BVH and
            # triangles stay in L2)
            "roofline": {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback",
                         "evidence": evidence,
                         "per_kernel": per_kernel,
                         "frame": {"alg_bytes": alg_frame, "achieved": alg_frame / (ms_per_step / 1e3) / 1e9}},
            "cpu_baseline": cpu,
        }
        if not args.no_legs:
            # the other two legs of the metric: batched vs plain, backward / forward
            line["batch"] = batch_leg(args.leg_steps, 1, clocks_index=local)
            line["diff"] = diff_leg(args.leg_steps, 2, clocks_index=local)
        print(json.dumps(line))
    ctx.close()
    replicas.finalize()


if __name__ == "__main__":
    main()
