"""Headless renderer of a scene file (bin/data/Scenes/*.json format): loads the
meshes (scene.py), ray casts the G-buffer and shadow map on the GPU
(gi_gbuffer_mesh, gi_shadow_map_mesh), computes the direct light and renders
the GI frame with the library's renderer, then writes the lit image.

  python -m legitengine_gb300.render_scene SCENE.json --out lit.pfm [--width 1280
      --height 720 --dirs 16 --cap 64 --bounces 2 --precision fast|texture|exact --learned]

The camera and light are the reference application's (main.cpp:164-172); the
image is written as PFM (float RGB) or, for a .ppm name, tone mapped to 8 bits
(x / (1 + x), then gamma 1 / 2.2).  Prints one JSON line with the timings.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def write_image(path: str, rgb: np.ndarray) -> None:
    """rgb: (H, W, 3) float, row 0 at the top."""
    h, w, _ = rgb.shape
    if path.lower().endswith(".ppm"):
        x = np.clip(rgb, 0.0, None)
        x = (x / (1.0 + x)) ** (1.0 / 2.2)
        data = np.clip(np.round(x * 255.0), 0, 255).astype(np.uint8)
        with open(path, "wb") as f:
            f.write(b"P6\n%d %d\n255\n" % (w, h))
            f.write(data.tobytes())
        return
    with open(path, "wb") as f:  # PFM: bottom row first, little-endian floats
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(np.ascontiguousarray(rgb[::-1], dtype="<f4").tobytes())


def read_pfm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = (int(t) for t in f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), dtype="<f4" if scale < 0 else ">f4")
    return data.reshape(h, w, 3)[::-1]


class SceneInputs:
    """The GPU input stages of a loaded scene for one view: G-buffer, shadow map,
    direct light (device tensors)."""

    def __init__(self, gi, torch, scene, width: int, height: int, cull: int = 1):
        from . import scene as S
        self.gi, self.torch = gi, torch
        self.mesh = gi.MeshDevice(scene)
        cam, light = S.reference_cameras(gi)
        self.view = gi.view_from_camera(cam, width, height)
        ss = scene.shadow_size
        self.light_view = gi.view_from_camera(light, ss, ss)
        f = dict(dtype=torch.float32, device="cuda")
        self.albedo = torch.empty((height, width, 4), **f)
        self.emissive = torch.empty((height, width, 4), **f)
        self.normal = torch.empty((height, width, 4), **f)
        self.moments = torch.empty((height, width, 2), **f)
        self.ndc = torch.empty((height, width, 1), **f)
        self.direct = torch.empty((height, width, 4), **f)
        self.shadow = torch.empty((ss, ss, 1), **f)
        self.cull = cull

    def compute(self):
        gi = self.gi
        gi.gbuffer_mesh(self.view, self.mesh, self.albedo, self.emissive, self.normal, self.moments, self.ndc,
                        cull=self.cull)
        gi.shadow_map_mesh(self.light_view, self.mesh, self.shadow, cull=self.cull)
        gi.direct_light(self.view, self.light_view, self.albedo, self.emissive, self.normal, self.ndc, self.shadow,
                        self.direct)


def render(path: str, width: int = 1280, height: int = 720, dirs: int = 16, cap: int = 64, bounces: int = 2,
           precision: str = "fast", learned: bool = False, weights: str | None = None, cull: int = 1):
    """Renders the scene file at `path`; returns (lit image (H, W, 4) numpy, info dict)."""
    import torch

    from . import gi
    from . import scene as S
    from . import train_reconstructor as tr
    t0 = time.perf_counter()
    sc = S.load_scene(path)
    t_load = time.perf_counter() - t0
    inp = SceneInputs(gi, torch, sc, width, height, cull)
    prec = {"texture": gi.GI_MARCH_TEXTURE, "fast": gi.GI_MARCH_FAST, "exact": gi.GI_MARCH_EXACT}[precision]
    r = gi.Renderer(width, height, dirs=dirs, step_cap=cap, bounces=bounces, bilateral=True, precision=prec)
    net = None
    if learned:
        net = gi.Mlp(seed=None)
        net.load(weights or tr.DEFAULT_WEIGHTS)
        r.set_learned(net, few_dirs=tr.DEFAULT_FEW_DIRS, few_step_dirs=tr.DEFAULT_FEW_STEP_DIRS)
    lit = torch.empty((height, width, 4), dtype=torch.float32, device="cuda")
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record()
    inp.compute()
    e1.record()
    r.render(inp.view, inp.albedo, inp.normal, inp.moments, inp.ndc, inp.direct, lit)
    e2.record()
    torch.cuda.synchronize()
    out = lit.cpu().numpy()
    info = {"scene": path, "width": width, "height": height, "objects": int(len(sc.objects)),
            "triangles": int(len(sc.triangles)), "load_s": t_load, "inputs_ms": e0.elapsed_time(e1),
            "gi_ms": e1.elapsed_time(e2), "method": "learned" if learned else f"plain R={dirs}",
            "bounces": bounces, "precision": precision}
    r.close()
    return out, info


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("scene")
    ap.add_argument("--out", default="lit.pfm")
    ap.add_argument("--width", type=int, default=1280)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--dirs", type=int, default=16)
    ap.add_argument("--cap", type=int, default=64)
    ap.add_argument("--bounces", type=int, default=2)
    ap.add_argument("--precision", choices=("texture", "fast", "exact"), default="fast")
    ap.add_argument("--learned", action="store_true")
    ap.add_argument("--weights", default=None)
    ap.add_argument("--two-sided", action="store_true", help="hit both faces of every triangle (no culling)")
    a = ap.parse_args(argv)
    out, info = render(a.scene, a.width, a.height, a.dirs, a.cap, a.bounces, a.precision, a.learned, a.weights,
                       cull=0 if a.two_sided else 1)
    write_image(a.out, out[..., :3])
    info["out"] = a.out
    print(json.dumps(info))
    return 0


if __name__ == "__main__":
    sys.exit(main())
