"""Trains and evaluates the learned reconstructor on the GPU, with the library's
own kernels only (input stages, march, features, MLP forward/backward, Adam).

Training frame f: seeded room (scene seed 4000 + f % scenes, 256 scenes; 64
boxes, 16 spheres), camera on spline 10000 + f // 64 at frame f % 64.  Per frame: the
G-buffer, shadow map and direct light; both pyramids; the few-ray march (R = 2)
and its mip levels 1-4; the plain method's many-ray gather (R = 256, no step
cap) on `tiles_per_frame` random march tiles as targets; the features of those
tiles; one Adam step on the batch (32 tiles x 2048 pixels = 65,536 pixels), each
pixel's absolute error (GI_MLP_LOSS_ABSOLUTE: the L1 error the evaluation measures)
weighted by its exposure scale over the batch mean.

Evaluation frames use scene seeds 20000+ and spline 20000 (never trained on).
The error of a method is the relative L1 distance, over all pixels and the rgb
channels, between its bilaterally filtered indirect light and the filtered
R = 256 gather of the same frame.

The committed networks were made with
  python -m legitengine_gb300.train_reconstructor --frames 2000 --few-dirs 1 --few-step-dirs 32 \
      --out legitengine_gb300/data/reconstructor_1dir.bin      (the default: 1 direction)
  python -m legitengine_gb300.train_reconstructor --frames 2000 --few-dirs 2 --few-step-dirs 32 \
      --out legitengine_gb300/data/reconstructor_2dir.bin      (2 directions)
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

PKG = Path(__file__).resolve().parent
sys.path.insert(0, str(PKG.parent))

DEFAULT_WEIGHTS = PKG / "data" / "reconstructor_1dir.bin"  # 1 direction stepped at 32-direction density
R2_WEIGHTS = PKG / "data" / "reconstructor_2dir.bin"  # 2 directions stepped at 32-direction density
DEFAULT_FEW_DIRS, DEFAULT_FEW_STEP_DIRS = 1, 32


class Frame:
    """Device buffers of one viewport: G-buffer, direct light, pyramids."""

    def __init__(self, gi, torch, W, H, shadow_size=1024):
        self.gi, self.torch, self.W, self.H = gi, torch, W, H
        f = dict(dtype=torch.float32, device="cuda")
        self.albedo = torch.empty((H, W, 4), **f)
        self.emissive = torch.empty((H, W, 4), **f)
        self.normal = torch.empty((H, W, 4), **f)
        self.moments = torch.empty((H, W, 2), **f)
        self.ndc = torch.empty((H, W, 1), **f)
        self.direct = torch.empty((H, W, 4), **f)
        self.shadow = torch.empty((shadow_size, shadow_size, 1), **f)
        self.L = gi.mip_level_count(W, H, 10)
        self.ll = [self.direct] + gi.alloc_pyramid(W, H, 4, self.L)[1:]
        self.dl = [self.moments] + gi.alloc_pyramid(W, H, 2, self.L)[1:]
        self.lb = [self.direct] + gi.alloc_pyramid(W, H, 4, self.L)[1:]
        self.db = [self.moments] + gi.alloc_pyramid(W, H, 2, self.L)[1:]
        self.few = gi.alloc_pyramid(W, H, 4, 5)
        self.few_f = torch.empty((H, W, 4), **f)
        self.tx, self.ty, self.tw, self.th = gi.march_tile_grid(W, H, 4)

    def inputs(self, prims_dev, nprims, view, light_view):
        gi = self.gi
        gi.gbuffer(view, prims_dev, nprims, self.albedo, self.emissive, self.normal, self.moments, self.ndc)
        gi.shadow_map(light_view, prims_dev, nprims, self.shadow)
        gi.direct_light(view, light_view, self.albedo, self.emissive, self.normal, self.ndc, self.shadow,
                        self.direct)
        gi.build_mips(self.ll, 4)
        gi.build_mips(self.dl, 2)
        gi.blur_pyramid(self.ll, self.lb)
        gi.blur_pyramid(self.dl, self.db)
        self.view = view

    def march(self, dirs, cap, out, tiles=None, step_dirs=0, precision=0):
        p = self.gi.GiMarchParams(dirs, cap, 4, step_dirs, precision)
        if tiles is None:
            self.gi.march(self.view, p, self.lb, self.db, self.normal, self.ndc, out)
        else:
            self.gi.march_tiles(self.view, p, self.lb, self.db, self.normal, self.ndc, out, tiles)

    def few_ray(self, dirs=2, cap=64, step_dirs=0, precision=0):
        self.march(dirs, cap, self.few[0], step_dirs=step_dirs, precision=precision)
        self.gi.build_mips(self.few, 4)
        self.gi.bilateral(self.few[0], self.moments, self.normal, self.few_f)

    def reconstruct(self, net, out):
        """Fused features + network (tensor cores) over the whole frame."""
        net.reconstruct(self.moments, self.normal, self.albedo, self.direct, [self.few[0], self.few[2], self.few[4]],
                        self.few_f, self.db[2], out)

    def features(self, out, scale, tiles=None):
        self.gi.features(self.moments, self.normal, self.albedo, self.direct,
                         [self.few[0], self.few[2], self.few[4]], self.few_f, self.db[2], out, scale, tiles=tiles)


def scene(gi, seed, boxes=64, spheres=16):
    prims = gi.scene_generate(seed, boxes, spheres)
    return gi.prims_to_device(prims)


def train(frames=2000, width=1920, height=1080, tiles_per_frame=32, few_dirs=2, target_dirs=256, lr=1e-3,
          scenes=256, seed=0, out=DEFAULT_WEIGHTS, log_every=100, mlp=None, verbose=True, lr_final=1e-4,
          few_step_dirs=0, loss="absolute"):
    """Cosine learning-rate decay from lr to lr_final over the frames.  loss: "absolute"
    (the weighted L1 error the evaluation measures; the shipped networks) or
    "squared" (clipped squared error)."""
    import math
    import torch
    from legitengine_gb300 import gi
    torch.cuda.set_device(0)
    fr = Frame(gi, torch, width, height)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    net = mlp if mlp is not None else gi.Mlp(seed=seed)
    net.set_loss(gi.GI_MLP_LOSS_ABSOLUTE if loss == "absolute" else gi.GI_MLP_LOSS_SQUARED)
    n_tiles = fr.tx * fr.ty
    g = torch.Generator(device="cpu").manual_seed(seed)
    tp = fr.tw * fr.th
    target_img = torch.zeros((height, width, 4), dtype=torch.float32, device="cuda")
    T = torch.empty((tiles_per_frame * tp, 4), dtype=torch.float32, device="cuda")
    X = torch.empty((tiles_per_frame * tp, 32), dtype=torch.bfloat16, device="cuda")
    S = torch.empty((tiles_per_frame * tp,), dtype=torch.float32, device="cuda")
    scenes_dev, scenes_host = {}, {}
    losses = []
    t0 = time.time()
    for f in range(frames):
        sseed = 4000 + f % scenes
        if sseed not in scenes_dev:
            scenes_host[sseed] = gi.scene_generate(sseed, 64, 16)
            scenes_dev[sseed] = gi.prims_to_device(scenes_host[sseed])
        pd, npr = scenes_dev[sseed]
        view = gi.view_from_camera(gi.camera_spline(10000 + f // 64, f % 64, 64, scenes_host[sseed]), width,
                                   height)
        fr.inputs(pd, npr, view, light)
        fr.few_ray(few_dirs, step_dirs=few_step_dirs)
        tiles = torch.randperm(n_tiles, generator=g)[:tiles_per_frame].to(torch.int32).cuda()
        fr.march(target_dirs, 0, target_img, tiles)
        gi.gather_tiles(target_img, tiles, T)
        fr.features(X, S, tiles)
        # Loss weight of a pixel: its exposure scale over the batch mean, so that the
        # error (in units of the scale) weighs pixels by their light the way the frame's
        # relative L1 error does.  Channel 3 of the gathered march output is 1
        # inside the image and 0 for the parts of edge tiles outside it.
        T[:, 3] *= S / S.mean()
        lr_f = lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * f / max(1, frames - 1)))
        loss = net.train_step(X, T, lr=lr_f, want_loss=(f % 10 == 0), scale=S)
        if loss is not None:
            losses.append((f, loss))
        if verbose and log_every and f % log_every == 0:
            print(f"frame {f:5d}  loss {loss if loss is not None else float('nan'):.5f}  {time.time() - t0:.1f}s",
                  flush=True)
    if out:
        Path(out).parent.mkdir(parents=True, exist_ok=True)
        net.save(out)
    return net, losses


def rel_l1(a, b):
    return float((a[..., :3] - b[..., :3]).abs().sum() / b[..., :3].abs().sum().clamp_min(1e-20))


def evaluate(net, frames=4, width=1920, height=1080, few_dirs=2, plain_dirs=(2, 4, 8, 16, 32), cap=64,
             ref_dirs=256, seed_base=20000, verbose=True, few_step_dirs=0, boxes=64, spheres=16, precision=0):
    """Error and cost of the plain method at each R in plain_dirs and of the learned method
    (few_dirs + MLP).  Error: relative L1 over pixels and rgb of the bilaterally filtered
    indirect light against the filtered R = ref_dirs gather without a step cap.  Cost: GPU
    milliseconds of the method's indirect-light passes for one bounce (CUDA events).  precision:
    the march precision of both methods (the R = ref_dirs reference is always exact)."""
    import torch
    from legitengine_gb300 import gi
    fr = Frame(gi, torch, width, height)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    f32 = dict(dtype=torch.float32, device="cuda")
    ref, ref_f, img, img_f = (torch.empty((height, width, 4), **f32) for _ in range(4))
    err = {f"plain{r}": [] for r in plain_dirs}
    err["learned"] = []
    err["few"] = []
    err["few_mip2"] = []
    ms = {k: [] for k in err}
    raw = {k: [] for k in err}  # the same results against the unfiltered R = ref_dirs gather

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fn()  # warm
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def learned():
        fr.few_ray(few_dirs, cap, step_dirs=few_step_dirs, precision=precision)
        fr.reconstruct(net, img)

    for k in range(frames):
        prims = gi.scene_generate(seed_base + k, boxes, spheres)
        pd, npr = gi.prims_to_device(prims)
        view = gi.view_from_camera(gi.camera_spline(seed_base, (k * 16) % 64, 64, prims), width, height)
        fr.inputs(pd, npr, view, light)
        fr.march(ref_dirs, 0, ref)
        gi.bilateral(ref, fr.moments, fr.normal, ref_f)
        for r in plain_dirs:
            ms[f"plain{r}"].append(timed(lambda: fr.march(r, cap, img, precision=precision)))
            gi.bilateral(img, fr.moments, fr.normal, img_f)
            err[f"plain{r}"].append(rel_l1(img_f, ref_f))
            raw[f"plain{r}"].append(rel_l1(img_f, ref))
        ms["learned"].append(timed(learned))
        err["learned"].append(rel_l1(img, ref_f))  # the network's blend replaces the filtered light
        raw["learned"].append(rel_l1(img, ref))
        ms["few"].append(0.0)
        gi.bilateral(fr.few[0], fr.moments, fr.normal, img_f)
        err["few"].append(rel_l1(img_f, ref_f))
        raw["few"].append(rel_l1(img_f, ref))
        # the mip-2 candidate alone (what the network gains over always taking it)
        up = torch.nn.functional.interpolate(fr.few[2].permute(2, 0, 1)[None], size=(height, width),
                                             mode="bilinear", align_corners=False)[0].permute(1, 2, 0)
        err["few_mip2"].append(rel_l1(up, ref_f))
        raw["few_mip2"].append(rel_l1(up, ref))
        ms["few_mip2"].append(0.0)
        if verbose:
            print(f"eval frame {k}: " + "  ".join(f"{n} {err[n][-1]:.4f}/{ms[n][-1]:.2f}ms" for n in err), flush=True)
    return {n: {"error": sum(v) / len(v), "ms": sum(ms[n]) / len(ms[n]),
                "error_vs_unfiltered": sum(raw[n]) / len(raw[n])} for n, v in err.items()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=2000)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--tiles", type=int, default=32)
    ap.add_argument("--few-dirs", type=int, default=DEFAULT_FEW_DIRS)
    ap.add_argument("--few-step-dirs", type=int, default=DEFAULT_FEW_STEP_DIRS)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-final", type=float, default=1e-4)
    ap.add_argument("--loss", choices=("absolute", "squared"), default="absolute")
    ap.add_argument("--out", default=str(DEFAULT_WEIGHTS))
    ap.add_argument("--eval-frames", type=int, default=4)
    ap.add_argument("--eval-json", default="")
    a = ap.parse_args()
    net, losses = train(a.frames, a.width, a.height, a.tiles, a.few_dirs, lr=a.lr, out=a.out,
                        few_step_dirs=a.few_step_dirs, lr_final=a.lr_final, loss=a.loss)
    print("final losses:", losses[-5:])
    if a.eval_frames:
        r = evaluate(net, a.eval_frames, a.width, a.height, a.few_dirs, few_step_dirs=a.few_step_dirs)
        print("eval:", r)
        if a.eval_json:
            import json
            Path(a.eval_json).write_text(json.dumps(r, indent=1))


if __name__ == "__main__":
    main()
