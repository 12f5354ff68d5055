#!/usr/bin/env python3
"""GI Mpix/s of the screen-space GI path at 1920x1080 on GB300.

Workload (plain method): seeded procedural room with 64 boxes and 16 spheres,
1920x1080, R = 16 directions per pixel, step cap 64, 2 bounces (bounce 2
marches over the light pyramid of bounce 1's gathered image), 5x5 bilateral,
over a 64-frame seeded camera spline.  One step = the GI passes of one frame
(mip chains, blur pyramids, march, bilateral, final gather, both bounces) on
G-buffer inputs already resident in HBM; the input stages (G-buffer, shadow
map, direct light) run before the timed region.  The 64 frames' inputs (7.9
GB) are cycled, so no step finds its inputs in the 129 MB L2.

`--impl reference` times the CPU restatement of the same path (the reference's
GLSL cannot run here: no Vulkan stack, and its renderer host does not build).

Prints ONE JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GI Mpix/s at 1080p on 1 GB300, learned vs plain at matched error vs FP64 oracle"
MARCH_BYTES_PER_PX = 60.0   # compulsory bytes of the march per pixel (normal 12, depth 4, pyramids 32, out 12)
SCENE_SEED = 2 * 1000 + 0   # configuration 2, scene 0
SPLINE_SEED = 2


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=64)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--dirs", type=int, default=16)
    p.add_argument("--cap", type=int, default=64)
    p.add_argument("--bounces", type=int, default=2)
    p.add_argument("--frames", type=int, default=64)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-learned", action="store_true")
    p.add_argument("--eval-frames", type=int, default=4)
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--no-learned-batched", action="store_true")
    p.add_argument("--no-soft", action="store_true")
    p.add_argument("--precision", choices=["texture", "fast", "exact"], default="texture",
                   help="march step-loop precision: texture (the fast loop with its depth and light taps fetched "
                        "by the texture units; its distance to exact is measured and reported), fast (software "
                        "taps, within 1e-3 of exact per pixel at 16 directions) or exact (bit-identical to the CPU "
                        "restatement)")
    return p.parse_args()


def workload(a):
    return {
        "workload": f"plain GI, {a.width}x{a.height}, 64 boxes + 16 spheres, R={a.dirs}, step cap {a.cap}, "
                    f"{a.bounces} bounces, 5x5 bilateral, {a.frames}-frame camera spline",
        "method": "plain",
        "width": a.width, "height": a.height, "dirs": a.dirs, "step_cap": a.cap, "bounces": a.bounces,
        "frames": a.frames, "mip_levels": 10, "pattern": 4, "march_precision": a.precision,
        "l2": f"inputs cycle over {a.frames} resident frames (~{a.frames * a.width * a.height * 60 / 1e9:.1f} GB) > L2",
    }


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def reference_inputs(a, n_frames: int = 2):
    """Input stages of the first frames on the host, built by the oracle alone
    (scene, light, cameras and view matrices restated there): the reference arm
    and the CPU baseline load nothing of the CUDA library."""
    from oracle import oracle as O
    prims = O.scene_generate(SCENE_SEED, 64, 16)
    light = O.view_from_camera(O.scene_light(), 1024, 1024)
    sm = O.shadow_map(light, prims)
    out = []
    for f in range(n_frames):
        view = O.view_from_camera(O.camera_spline(SPLINE_SEED, f, a.frames), a.width, a.height)
        gb = O.gbuffer(view, prims)
        out.append((view, gb, O.direct_light(view, light, gb, sm)))
    return out


def reference_frame(a, inputs):
    """One whole frame of the GI path on the host cores (all threads): the
    oracle's restatement in the reference's own float evaluation (the C library's
    functions, true division, glm's operation order -- bit-identical to the
    reference's GLSL compiled as C++ given the shader's matrices, as
    tests/test_ref_pin.py checks): mip chains, blur pyramids, the R-direction
    march, bilateral and gather, every bounce.  Returns seconds."""
    from oracle import oracle as O
    view, gb, direct = inputs
    O.set_libm(True)
    try:
        t0 = time.perf_counter()
        O.render_frame(view, gb, direct, a.dirs, a.cap, bounces=a.bounces)
        return time.perf_counter() - t0
    finally:
        O.set_libm(False)


def cpu_baseline(a):
    """The same workload on the host cores: one whole frame (about 10-30 s)."""
    from oracle import oracle as O
    inputs = reference_inputs(a, 1)[0]
    dt = reference_frame(a, inputs)
    return {"value": a.width * a.height / dt / 1e6, "unit": "Mpix/s", "cores": O.threads(), "kind": "port",
            "sample": f"one whole {a.width}x{a.height} frame ({a.bounces} bounces, R={a.dirs}): {dt:.1f} s"}


# ---------------------------------------------------------------------------
def run_reference(a, rank):
    """The reference's path on the host cores: every step one whole frame (the
    frames alternate between two precomputed G-buffers; the input stages run
    before the timed steps, as in the GPU arm)."""
    if rank != 0:
        return
    from oracle import oracle as O
    frames = reference_inputs(a, 2)
    times = []
    # One warm-up frame at most: the host path has no compilation or clock ramp to
    # wait out, and a frame takes ~11 s on 16 cores.
    warm = min(a.warmup, 1)
    for i in range(warm + a.steps):
        dt = reference_frame(a, frames[i % len(frames)])
        if i >= warm:
            times.append(dt)
    total = sum(times)
    v = a.width * a.height * a.steps / total / 1e6
    out = {
        "metric": METRIC, "value": v, "unit": "Mpix/s", "impl": "reference", "n_gpus": a.gpus, "steps": a.steps,
        "warmup": warm, "ms_per_step": total / a.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload(a),
        "cpu_baseline": {"value": v, "unit": "Mpix/s", "cores": O.threads(), "kind": "port",
                         "sample": f"{a.steps} whole {a.width}x{a.height} frames, one per step"},
        "e2e": {"value": v, "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's GLSL passes as the oracle restates them, in the reference's float evaluation "
                "(bit-identical to its shaders compiled as C++, tests/test_ref_pin.py); its own renderer needs "
                "Vulkan and an absent submodule",
    }
    print(json.dumps(out), flush=True)


def traffic_from_profile(name: str):
    """Per-launch DRAM bytes of a kernel from its committed ncu summary (profiles/<name>.txt)."""
    p = ROOT / "profiles" / f"{name}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch_full_frame:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def issue_from_profile(name: str):
    """Issue-side figures of a kernel from its committed ncu summary (profiles/<name>.txt):
    the share of issue slots busy and the DRAM throughput, for the bound the HBM roofline
    cannot show."""
    p = ROOT / "profiles" / f"{name}.txt"
    if not p.exists():
        return None
    out = {"source": f"profiles/{name}.txt"}
    for line in p.read_text().splitlines():
        for key, label in (("issue_slots_busy_pct", "Issue slots busy"), ("dram_throughput_pct", "DRAM throughput")):
            if line.startswith(label):
                try:
                    out[key] = float(line[len(label):].split()[0])
                except ValueError:
                    pass
    return out


def pass_profile(r, torch, stream, render_one, frames=8):
    """Extra frames (outside any timed region) with the renderer's per-pass GPU
    profiler on: milliseconds per pass name (summed over bounces) and per frame,
    the mean over `frames` frames after one untimed.  render_one(k) renders the
    k-th of them (views spread over the timed loop's, whose cost varies by view)."""
    r.set_profiling(True)
    out = {}
    for k in range(frames + 1):
        with torch.cuda.stream(stream):
            render_one(max(0, k - 1))
        stream.synchronize()
        if k == 0:
            continue
        times = r.pass_times()
        for name, t0, t1 in times:
            out[name] = out.get(name, 0.0) + (t1 - t0) / frames
        out["frame"] = out.get("frame", 0.0) + (times[-1][2] if times else 0.0) / frames
    r.set_profiling(False)
    return {k: round(v, 4) for k, v in out.items()}


def learned_leg(a, gi, torch, frames, stream, lit, plain_value):
    """The learned method on the same frames (1 direction stepped at 32 + the reconstructor,
    judge on 1/64 of the tiles), and its error against the converged R=256 gather next to the
    plain method's error-vs-cost curve."""
    import math
    from legitengine_gb300 import train_reconstructor as tr
    W, H, F = a.width, a.height, a.frames
    net = gi.Mlp(seed=None)
    net.load(tr.DEFAULT_WEIGHTS)
    r = gi.Renderer(W, H, dirs=a.dirs, step_cap=a.cap, bounces=a.bounces, bilateral=True, precision=PREC[a.precision])
    r.set_learned(net, few_dirs=tr.DEFAULT_FEW_DIRS, few_step_dirs=tr.DEFAULT_FEW_STEP_DIRS, judge_every=64,
                  threshold=0.25)

    def step(i):
        view, t = frames[i % F]
        r.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit)

    with torch.cuda.stream(stream):
        for i in range(a.warmup):
            step(i)
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        torch.cuda.nvtx.range_push("learned_timed")
        e0.record(stream)
        for i in range(a.steps):
            step(a.warmup + i)
        e1.record(stream)
        torch.cuda.nvtx.range_pop()
    stream.synchronize()
    ms = e0.elapsed_time(e1)
    judged, fell = r.stats()
    passes = pass_profile(r, torch, stream, lambda k: step(k * max(1, F // 8)))
    value = W * H * a.steps / (ms / 1e3) / 1e6
    ev = tr.evaluate(net, frames=a.eval_frames, width=W, height=H, few_dirs=tr.DEFAULT_FEW_DIRS,
                     few_step_dirs=tr.DEFAULT_FEW_STEP_DIRS, verbose=False, precision=PREC[a.precision])
    def matched(key):
        """The plain gather's cost at the learned error (log-log interpolation of its curve)."""
        pts = sorted(((v[key], v["ms"]) for k, v in ev.items() if k.startswith("plain")), key=lambda p: p[1])
        le = ev["learned"][key]
        for (ea, ma), (eb, mb) in zip(pts[:-1], pts[1:]):
            if (ea - le) * (eb - le) <= 0 and ea != eb:
                f = (math.log(le) - math.log(ea)) / (math.log(eb) - math.log(ea))
                return math.exp(math.log(ma) + f * (math.log(mb) - math.log(ma)))
        return None

    # The reconstruction's tensor-core roofline: 20,864 FLOP of network per pixel (2 x the four
    # layers' multiply-adds, the head's 3 outputs) per launch, one launch per bounce, timed by the
    # pass profiler, against the measured sustained bf16 rate (a kernel inside a long step).
    recon = None
    rec_ms = passes.get("ReconstructPass") if passes else None
    if rec_ms:
        try:
            peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        except (OSError, ValueError):
            peaks = {}
        peak = float(peaks.get("bf16_tflops_sustained", 1700.0))
        flop = 20864.0 * W * H
        launch_ms = rec_ms / a.bounces
        achieved = flop / (launch_ms / 1e3) / 1e12
        recon = {"bound": "tensor", "kernel": "mlp_reconstruct_kernel (features + network, tcgen05)",
                 "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                 "flop_per_px": 20864, "launch_ms": launch_ms,
                 "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained" if "bf16_tflops_sustained" in peaks
                 else "fallback 1700 TFLOP/s"}
    le, lm = ev["learned"]["error"], ev["learned"]["ms"]
    matched_ms = matched("error")
    matched_raw = matched("error_vs_unfiltered")
    lr = ev["learned"]["error_vs_unfiltered"]
    return {
        "value": value, "unit": "Mpix/s", "ms_per_step": ms / a.steps,
        "method": "1 direction stepped at 32-direction density + 32-64-64-64-3 reconstructor on the tcgen05 "
                  "tensor cores (features fused; softmax blend of the bilaterally filtered few-ray light and its "
                  "mip-2 and mip-4 averages), judge: plain R=16 on 1/64 of tiles, threshold 0.25",
        "throughput_vs_plain": value / plain_value,
        "error": le, "plain_error": ev[f"plain{a.dirs}"]["error"] if f"plain{a.dirs}" in ev else None,
        "error_metric": "relative L1 (rgb, all pixels) of the bounce-1 indirect light after filtering, against the "
                        "bilaterally filtered R=256 gather without a step cap; mean over held-out frames",
        "eval_frames": a.eval_frames,
        "plain_curve": {k: v for k, v in ev.items() if k.startswith("plain")},
        "learned_ms_per_bounce": lm,
        "plain_ms_at_matched_error": matched_ms,
        "speedup_at_matched_error": (matched_ms / lm) if matched_ms else None,
        "judged_tiles": judged, "fallback_tiles": fell,
        "few_ray_filtered_error": ev["few"]["error"],
        "mip2_candidate_error": ev["few_mip2"]["error"],
        "network_gain_over_mip2_candidate": ev["few_mip2"]["error"] / le if le else None,
        "against_unfiltered_reference": {
            "note": "the same results against the unfiltered R=256 gather without a step cap (exact contract; "
                    "its FP32 and FP64 evaluations agree to < 1e-3)",
            "learned": lr, "mip2_candidate": ev["few_mip2"]["error_vs_unfiltered"],
            "few_ray_filtered": ev["few"]["error_vs_unfiltered"],
            "plain_curve": {k: v["error_vs_unfiltered"] for k, v in ev.items() if k.startswith("plain")},
            "network_gain_over_mip2_candidate": ev["few_mip2"]["error_vs_unfiltered"] / lr if lr else None,
            "speedup_at_matched_error": (matched_raw / lm) if matched_raw else None,
        },
        "reconstruct_roofline": recon,
        "pass_ms": passes,
    }


PREC = {"exact": 0, "fast": 1, "texture": 2}

BATCH_RES = [(256, 256), (640, 480), (1280, 720), (1920, 1080), (2048, 1152)]


def batched_leg(gi, torch, steps=16, warmup=3, views=32, seed=3, precision=0):
    """32 independent seeded scenes (16-128 primitives) at resolutions drawn from
    BATCH_RES with 8-32 directions each, one bounce: every view's pyramids, one
    persistent march launch over all views, bilateral and gather, replayed as one
    CUDA graph (gi_batch_*).  Mpix/s = pixels of all views / frame time."""
    import numpy as np
    rng = np.random.RandomState(seed)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    f = dict(dtype=torch.float32, device="cuda")
    shadow = torch.empty((1024, 1024, 1), **f)
    specs, pix, desc = [], 0, []
    for i in range(views):
        W, H = BATCH_RES[rng.randint(len(BATCH_RES))]
        R = int(rng.randint(8, 33))
        n = int(rng.randint(16, 129))
        spheres = n // 5
        prims = gi.scene_generate(3000 + i, n - spheres, spheres)
        pd, npr = gi.prims_to_device(prims)
        view = gi.view_from_camera(gi.camera_spline(3000 + i, 0, 64, prims), W, H)
        t = {k: torch.empty((H, W, c), **f) for k, c in (("albedo", 4), ("emissive", 4), ("normal", 4),
                                                         ("moments", 2), ("ndc", 1), ("direct", 4), ("out_lit", 4))}
        gi.gbuffer(view, pd, npr, t["albedo"], t["emissive"], t["normal"], t["moments"], t["ndc"])
        gi.shadow_map(light, pd, npr, shadow)
        gi.direct_light(view, light, t["albedo"], t["emissive"], t["normal"], t["ndc"], shadow, t["direct"])
        specs.append(dict(view=view, march=gi.GiMarchParams(R, 64, 4, 0, precision), **t))
        pix += W * H
        desc.append(f"{W}x{H}/R{R}/{n}p")
    torch.cuda.synchronize()
    b = gi.Batch(specs, tile_rows=0)
    info = b.info()
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    for _ in range(warmup):
        b.render(sp)
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("batched_timed")
    e0.record(stream)
    for _ in range(steps):
        b.render(sp)
    e1.record(stream)
    torch.cuda.nvtx.range_pop()
    stream.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # The same views rendered one by one through the single-view renderer, for comparison.
    single_ms = 0.0
    rs = []
    for s in specs:
        W, H = s["view"].width, s["view"].height
        rs.append(gi.Renderer(W, H, dirs=s["march"].dirs, step_cap=64, bounces=1, bilateral=True,
                              precision=precision))
    with torch.cuda.stream(stream):
        for _ in range(2):
            for r, s in zip(rs, specs):
                r.render(s["view"], s["albedo"], s["normal"], s["moments"], s["ndc"], s["direct"], s["out_lit"])
        e0.record(stream)
        for _ in range(3):
            for r, s in zip(rs, specs):
                r.render(s["view"], s["albedo"], s["normal"], s["moments"], s["ndc"], s["direct"], s["out_lit"])
        e1.record(stream)
    stream.synchronize()
    single_ms = e0.elapsed_time(e1) / 3
    for r in rs:
        r.close()
    b.close()
    return {"value": pix / (ms / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_step": ms, "views": views,
            "pixels_per_step": pix, "steps": steps, "warmup": warmup, "tile_rows": info["tile_rows"],
            "work_items": info["work_items"], "grid": info["grid"],
            "one_by_one_ms": single_ms, "speedup_vs_one_by_one": single_ms / ms,
            "workload": "32 seeded scenes (16-128 primitives) at resolutions from {256^2, 640x480, 1280x720, "
                        "1920x1080, 2048x1152}, R 8-32, step cap 64, 1 bounce, 5x5 bilateral, one captured launch",
            "views_desc": desc}


def learned_batched_leg(gi, torch, steps=32, warmup=3, views=8, W=3840, H=2160, finetune_every=16, precision=0):
    """8 views at 3840x2160 of seeded rooms with 256 boxes and 64 spheres in one batch:
    the plain 32-direction gather, then the learned form (1 direction stepped at 32 +
    the reconstructor, judge on 1/64 of the tiles, fine-tuned every 16 frames on the
    judged tiles against a 256-direction march).  Errors of both forms against the
    converged 256-direction gather on a held-out 4K frame of the same scene type."""
    from legitengine_gb300 import train_reconstructor as tr
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    f = dict(dtype=torch.float32, device="cuda")
    shadow = torch.empty((1024, 1024, 1), **f)
    specs = []
    for i in range(views):
        prims = gi.scene_generate(5000 + i, 256, 64)
        pd, npr = gi.prims_to_device(prims)
        view = gi.view_from_camera(gi.camera_spline(5000 + i, 0, 64, prims), W, H)
        t = {k: torch.empty((H, W, c), **f) for k, c in (("albedo", 4), ("emissive", 4), ("normal", 4),
                                                         ("moments", 2), ("ndc", 1), ("direct", 4), ("out_lit", 4))}
        gi.gbuffer(view, pd, npr, t["albedo"], t["emissive"], t["normal"], t["moments"], t["ndc"])
        gi.shadow_map(light, pd, npr, shadow)
        gi.direct_light(view, light, t["albedo"], t["emissive"], t["normal"], t["ndc"], shadow, t["direct"])
        del t["emissive"]
        specs.append(dict(view=view, march=gi.GiMarchParams(32, 64, 4, 0, precision), **t))
    torch.cuda.synchronize()
    b = gi.Batch(specs, tile_rows=0)
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    pix = views * W * H
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(n, fn):
        e0.record(stream)
        for i in range(n):
            fn(i)
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / n

    for _ in range(2):
        b.render(sp)
    plain_ms = timed(3, lambda i: b.render(sp))
    net = gi.Mlp(seed=None)
    net.load(tr.DEFAULT_WEIGHTS)
    net.set_loss(gi.GI_MLP_LOSS_ABSOLUTE)  # fine-tuning continues the shipped network's training loss
    b.set_learned(net, few_dirs=tr.DEFAULT_FEW_DIRS, few_step_dirs=tr.DEFAULT_FEW_STEP_DIRS, judge_every=64,
                  threshold=0.25)
    for _ in range(warmup):
        b.render(sp)
    stream.synchronize()
    learned_ms = timed(steps, lambda i: b.render(sp))
    sampled, losses = [], []

    def frame_ft(i):
        b.render(sp)
        if (i + 1) % finetune_every == 0:
            loss, err = b.finetune(net, target_dirs=256, lr=1e-5, stream=sp)
            losses.append(loss)
            sampled.append(err)

    torch.cuda.nvtx.range_push("learned_batched_timed")
    ft_ms = timed(steps, frame_ft)
    torch.cuda.nvtx.range_pop()
    judged, fell = b.stats()
    b.close()
    del specs
    torch.cuda.empty_cache()
    ev = tr.evaluate(net, frames=1, width=W, height=H, few_dirs=tr.DEFAULT_FEW_DIRS, plain_dirs=(32,),
                     few_step_dirs=tr.DEFAULT_FEW_STEP_DIRS, boxes=256, spheres=64, seed_base=5100, verbose=False,
                     precision=precision)
    return {"value": pix / (ft_ms / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_step": ft_ms, "steps": steps,
            "warmup": warmup, "views": views, "width": W, "height": H,
            "learned_mpix_s_without_finetune": pix / (learned_ms / 1e3) / 1e6,
            "plain32_mpix_s": pix / (plain_ms / 1e3) / 1e6, "plain32_ms_per_step": plain_ms,
            "speedup_vs_plain32": plain_ms / ft_ms,
            "finetune_every": finetune_every, "finetune_sampled_error": sampled, "finetune_loss": losses,
            "judged_tiles": judged, "fallback_tiles": fell, "fallback_rate": fell / judged if judged else None,
            "error_learned_4k": ev["learned"]["error"], "error_plain32_4k": ev["plain32"]["error"],
            "error_metric": "relative L1 (rgb) against the filtered 256-direction gather, one held-out 4K frame "
                            "(scene seed 5100, 256 boxes + 64 spheres); the fine-tuning error is on the judged "
                            "tiles of the last frame against their 256-direction march",
            "workload": "8 views 3840x2160, seeded rooms with 256 boxes + 64 spheres, plain R=32 / learned 1 "
                        "direction stepped at 32 + reconstructor, judge 1/64 of tiles, 1 bounce, one captured "
                        "launch per frame, fine-tuning every 16 frames (inside the timed region)"}


def streaming_leg(gi, torch, hbm_peak, W=1920, H=1080, reps=10):
    """The HBM-streaming passes of the frame at 1920x1080, one launch at a time with
    L2 flushed in between (a 256 MB write), CUDA events around each launch:
    compulsory bytes of this library's layouts (fp32; light, normal and outputs 4
    channels, depth moments 2) / median launch time, against the measured HBM peak."""
    f = dict(dtype=torch.float32, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(7)
    img = lambda c: torch.rand((H, W, c), generator=g, **f) + 0.1
    direct, ind, albedo, normal, out = img(4), img(4), img(4), img(4), img(4)
    moments = img(2)
    L = gi.mip_level_count(W, H, 10)
    ll, dl = [direct] + gi.alloc_pyramid(W, H, 4, L)[1:], [moments] + gi.alloc_pyramid(W, H, 2, L)[1:]
    lb, db = [direct] + gi.alloc_pyramid(W, H, 4, L)[1:], [moments] + gi.alloc_pyramid(W, H, 2, L)[1:]
    gi.build_mips(ll, 4)
    gi.build_mips(dl, 2)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    third = sum((W >> k) * (H >> k) for k in range(1, L)) / (W * H)  # the levels >= 1 per level-0 pixel
    passes = {
        "mip_chain_light": (lambda: gi.build_mips(ll, 4), 16 + 16 * third),
        "mip_chain_depth": (lambda: gi.build_mips(dl, 2), 8 + 8 * third),
        "blur_pyramids": (lambda: (gi.blur_pyramid(ll, lb), gi.blur_pyramid(dl, db)), 2 * (16 + 8) * third),
        "bilateral_5x5": (lambda: gi.bilateral(ind, moments, normal, out), 16 + 8 + 16 + 16),
        "deinterleave_4ch": (lambda: gi.deinterleave(direct, out), 32),
        "interleave_4ch": (lambda: gi.interleave(out, ind), 32),
        "final_gather": (lambda: gi.final_gather(direct, ind, albedo, out), 16 * 4),
        # context, not a pass of the library: a device-to-device copy of one 4-channel image
        "torch_copy_4ch": (lambda: out.copy_(direct), 32),
    }
    res = {}
    for name, (fn, bpp) in passes.items():
        fn()
        ts = []
        for _ in range(reps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        ms = sorted(ts)[len(ts) // 2]
        gbs = bpp * W * H / (ms / 1e3) / 1e9
        res[name] = {"bytes_per_px": round(bpp, 3), "ms": round(ms, 5), "gbs": round(gbs, 1),
                     "frac": round(gbs / hbm_peak, 3)}
    res["note"] = ("L2 flushed before every launch; median of %d launches; peak = measured HBM copy bandwidth; "
                   "torch_copy_4ch = a plain device copy of the same size for comparison" % reps)
    return res


def soft_leg(gi, torch, W=1920, H=1080, frames=2):
    """The depth-variance (soft-occlusion) horizon against the reference's hard
    test at R = 8 and 16 (exact contract): error of each, bilaterally filtered,
    against the filtered 256-direction hard gather, and its march time."""
    from legitengine_gb300.train_reconstructor import Frame, rel_l1
    fr = Frame(gi, torch, W, H)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    f32 = dict(dtype=torch.float32, device="cuda")
    ref, ref_f, img, img_f = (torch.empty((H, W, 4), **f32) for _ in range(4))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    res = {}
    for k in range(frames):
        prims = gi.scene_generate(20000 + k, 64, 16)
        pd, npr = gi.prims_to_device(prims)
        fr.inputs(pd, npr, gi.view_from_camera(gi.camera_spline(20000, (k * 16) % 64, 64, prims), W, H), light)
        fr.march(256, 0, ref)
        gi.bilateral(ref, fr.moments, fr.normal, ref_f)
        for R in (8, 16):
            for occ, name in ((gi.GI_OCCLUSION_HARD, "hard"), (gi.GI_OCCLUSION_SOFT, "soft")):
                p = gi.GiMarchParams(R, 64, 4, 0, gi.GI_MARCH_EXACT, occ)
                gi.march(fr.view, p, fr.lb, fr.db, fr.normal, fr.ndc, img)
                e0.record()
                gi.march(fr.view, p, fr.lb, fr.db, fr.normal, fr.ndc, img)
                e1.record()
                torch.cuda.synchronize()
                gi.bilateral(img, fr.moments, fr.normal, img_f)
                r = res.setdefault(f"{name}{R}", {"error": 0.0, "ms": 0.0})
                r["error"] += rel_l1(img_f, ref_f) / frames
                r["ms"] += e0.elapsed_time(e1) / frames
    res["error_metric"] = ("relative L1 (rgb) of the filtered result against the filtered 256-direction hard "
                           f"gather, mean over {frames} held-out 1080p frames; ms = one march launch (exact contract)")
    return res


def max_over_ranks(ms: float, device: str) -> float:
    """The job's time: the slowest rank's, under torch.distributed; ms itself alone."""
    import torch
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_value(pixels_per_step: int, steps: int, world: int, ms: float) -> float:
    """Whole-job Mpix/s: every replica renders its own frames (weak scaling)."""
    return pixels_per_step * steps * world / (ms / 1e3) / 1e6


def run_ours(a, rank, world):
    import torch
    from legitengine_gb300 import gi

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    W, H, F = a.width, a.height, a.frames
    prims = gi.scene_generate(SCENE_SEED, 64, 16)
    pd, npr = gi.prims_to_device(prims)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    stream = torch.cuda.Stream()
    frames = []
    with torch.cuda.stream(stream):
        sm = torch.empty((1024, 1024, 1), dtype=torch.float32, device="cuda")
        gi.shadow_map(light, pd, npr, sm)
        for f in range(F):
            view = gi.view_from_camera(gi.camera_spline(SPLINE_SEED, f + rank * 7, F), W, H)
            t = {k: torch.empty((H, W, c), dtype=torch.float32, device="cuda")
                 for k, c in (("albedo", 4), ("emissive", 4), ("normal", 4), ("moments", 2), ("ndc", 1),
                              ("direct", 4))}
            gi.gbuffer(view, pd, npr, t["albedo"], t["emissive"], t["normal"], t["moments"], t["ndc"])
            gi.direct_light(view, light, t["albedo"], t["emissive"], t["normal"], t["ndc"], sm, t["direct"])
            del t["emissive"]
            frames.append((view, t))
    stream.synchronize()
    r = gi.Renderer(W, H, dirs=a.dirs, step_cap=a.cap, bounces=a.bounces, bilateral=True, precision=PREC[a.precision])
    lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")

    def step(i):
        view, t = frames[i % F]
        r.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit)

    with torch.cuda.stream(stream):
        for i in range(a.warmup):
            step(i)
    stream.synchronize()
    dist = world > 1
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    n0 = gi.lib().gi_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        torch.cuda.nvtx.range_push("plain_timed")
        e0.record(stream)
        for i in range(a.steps):
            step(a.warmup + i)
        e1.record(stream)
        torch.cuda.nvtx.range_pop()
    stream.synchronize()
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches = gi.lib().gi_launch_count() - n0
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), "cuda")
    passes_plain = pass_profile(r, torch, stream, lambda k: step(k * max(1, F // 8)))
    # The same frames with the bit-identical (exact) march, for reference.
    exact = None
    if a.precision != "exact":
        rx = gi.Renderer(W, H, dirs=a.dirs, step_cap=a.cap, bounces=a.bounces, bilateral=True,
                         precision=PREC["exact"])
        nx = min(16, a.steps)
        with torch.cuda.stream(stream):
            for i in range(3):
                view, t = frames[i % F]
                rx.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit)
            x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            x0.record(stream)
            for i in range(nx):
                view, t = frames[(3 + i) % F]
                rx.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit)
            x1.record(stream)
        stream.synchronize()
        xms = x0.elapsed_time(x1) / nx
        # The headline precision's distance to exact on the same frames.
        dist_l1, dist_max, dist_over = [], [], []
        lx = torch.empty_like(lit)
        with torch.cuda.stream(stream):
            for f in range(min(4, F)):
                view, t = frames[f]
                rx.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lx)
                r.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit)
                x, y = lit[..., :3].double(), lx[..., :3].double()
                rel = (x - y).abs() / torch.clamp(y.abs(), min=1e-3 * float(y.abs().mean()))
                dist_l1.append(float((x - y).abs().sum() / y.abs().sum()))
                dist_max.append(float(rel.max()))
                dist_over.append(float((rel > 1e-2).double().mean()))
        stream.synchronize()
        exact = {"value": W * H / (xms / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_step": xms, "steps": nx,
                 "march_precision": "exact (bit-identical to the CPU restatement)",
                 "headline_vs_exact": {"precision": a.precision, "frame_rel_l1": max(dist_l1),
                                       "max_rel": max(dist_max), "fraction_over_1e-2": max(dist_over),
                                       "frames": len(dist_l1),
                                       "note": "lit image, rgb; relative error floored at 1e-3 of the mean"}}
        rx.close()
    # Temporal feedback: one march per frame over the previous frame's gathered image.
    feedback = None
    if world == 1:
        rf = gi.Renderer(W, H, dirs=a.dirs, step_cap=a.cap, bounces=1, bilateral=True, precision=PREC[a.precision],
                         feedback=True)
        nf = min(16, a.steps)
        with torch.cuda.stream(stream):
            for i in range(3):
                view, t = frames[i % F]
                rf.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit)
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            for i in range(nf):
                view, t = frames[(3 + i) % F]
                rf.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit)
            f1.record(stream)
        stream.synchronize()
        fms = f0.elapsed_time(f1) / nf
        feedback = {"value": W * H / (fms / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_step": fms, "steps": nf,
                    "mode": "one march per frame over the previous frame's gathered image (bounces accumulate "
                            "over the spline's frames)"}
        rf.close()
    value = job_value(W * H, a.steps, world, ms)

    # Dominant kernels: the headline frame's own march launches -- bounce 1's
    # recording march and bounce 2's replay of its record -- timed by the
    # renderer's pass profiler (events around each IndirectLightPass, on the
    # renderer's stream) on the same renderer and frames as the timed loop.
    march_ms, replay_ms = [], []
    r.set_profiling(True)
    for i in range(3 + max(8, a.steps // 2)):
        view, t = frames[i % F]
        with torch.cuda.stream(stream):
            r.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit)
        stream.synchronize()
        ind = [t1 - t0 for name, t0, t1 in r.pass_times() if name == "IndirectLightPass"]
        if i >= 3:
            march_ms.append(ind[0])
            replay_ms.append(sum(ind[1:]))
    r.set_profiling(False)
    m_avg, r_avg = sum(march_ms) / len(march_ms), sum(replay_ms) / len(replay_ms)
    march_avg = (m_avg + r_avg) / a.bounces  # per launch: one march or replay per bounce
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = MARCH_BYTES_PER_PX * W * H / (march_avg / 1e3) / 1e9
    march_profile = f"march_headline_1080p_r16_{a.precision}"
    traffic = traffic_from_profile(march_profile)

    # End to end through the public host-buffer entry point (pinned host memory).
    e2e = None
    if True:  # every rank: the end-to-end figure is a whole-job number too
        # Every second frame of the spline in pinned host memory (124 MB of inputs each), so that the
        # end-to-end loop renders the same mix of views as the device-resident one.
        stride = 2 if F >= 8 else 1
        hf = []
        for f in range(0, F, stride):
            view, t = frames[f]
            hf.append((view, [t[k].cpu().pin_memory() for k in ("albedo", "normal", "moments", "ndc", "direct")]))
        # One pinned output per in-flight frame (the pipelined call keeps two frames in flight).
        hout = [torch.empty((H, W, 4), dtype=torch.float32).pin_memory() for _ in range(2)]
        sp = C.c_void_p(stream.cuda_stream)
        # Warm-up: one pass over every pinned frame, so that no buffer is first touched by a copy
        # inside the timed loop.
        for i in range(len(hf)):
            r.render_host_async(hf[i][0], *hf[i][1], hout[i % 2], stream=sp)
        r.host_wait()
        ne = max(4, len(hf), a.steps // 2)
        # The loop is timed on the host clock, which the box's other work disturbs by a few per cent
        # from one pass to the next: three passes, the median reported, every pass listed.
        passes_ms = []
        for _ in range(3):
            if dist:
                torch.distributed.barrier()
            t0 = time.perf_counter()
            for i in range(ne):  # each step: its inputs in, its lit image out, overlapped with the neighbours' rendering
                r.render_host_async(hf[i % len(hf)][0], *hf[i % len(hf)][1], hout[i % 2], stream=sp)
            r.host_wait()
            passes_ms.append(max_over_ranks((time.perf_counter() - t0) * 1e3, "cuda"))
        dt_ms = sorted(passes_ms)[1]
        h2d = sum(x.numel() * 4 for x in hf[0][1])
        e2e = {"value": job_value(W * H, ne, world, dt_ms), "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": hout[0].numel() * 4,
               "api": "gi_renderer_render_host_async (copies of frame k overlap the rendering of k - 1 / k + 1)",
               "frames": f"{len(hf)} pinned frames (every {stride} of the {F}-frame spline), cycled over {ne} steps",
               "passes_ms": [round(x, 3) for x in passes_ms], "reported": "median of the three passes"}

    learned = None
    if world == 1 and not a.no_learned:
        learned = learned_leg(a, gi, torch, frames, stream, lit, value)

    batched = None
    if world == 1 and not a.no_batched:
        batched = batched_leg(gi, torch, precision=PREC[a.precision])

    soft = None
    if world == 1 and not a.no_soft:
        soft = soft_leg(gi, torch)
    streaming = streaming_leg(gi, torch, hbm_peak) if world == 1 else None

    learned_batched = None
    if world == 1 and not a.no_learned_batched and not a.no_learned:
        learned_batched = learned_batched_leg(gi, torch, precision=PREC[a.precision])

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        cpu = cpu_baseline(a)

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded procedural room and camera spline (no dataset)",
            "config": workload(a) | {"parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "kernel": "march_kernel (recording) + march_replay_kernel",
                         "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                         "traffic": traffic, "avg_launch_ms": march_avg, "bytes_per_px": MARCH_BYTES_PER_PX,
                         "launches_per_step": a.bounces, "record_march_ms": m_avg, "replay_ms": r_avg,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback",
                         "note": "the headline frame's march launches (bounce 1 marches and records, bounce 2 "
                                 "re-lights the record), each credited with the march's 60 compulsory bytes per "
                                 "pixel; timed by the renderer's pass profiler on the timed loop's renderer and "
                                 "frames; traffic = DRAM bytes per launch from the committed ncu summary.  The "
                                 "march is bound by instruction issue and the latency of its dependent fetches "
                                 "(its working set lives in L2), so its HBM fraction is small by construction",
                         "issue": issue_from_profile(march_profile)},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk,
            # The large sub-objects, the ones read most last (a log keeps a line's end).
            "streaming_passes": streaming, "soft_occlusion": soft, "batched": batched,
            "learned_batched": learned_batched, "temporal_feedback": feedback, "pass_ms": passes_plain,
            "plain_exact": exact, "learned": learned,
        }
        print(json.dumps(out), flush=True)


def main():
    a = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    run_ours(a, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
