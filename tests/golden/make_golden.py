"""Writes tests/golden/kat.json: known answers derived directly from the
reference's formulas, in plain Python (neither the CUDA library nor the oracle is
used), so that the CPU tests can pin the oracle and the library against them.

Sources (paths inside the reference project):
  hammersley     bin/data/Shaders/glsl/SSVGI/indirectLighting.frag:102-112 (HammersleyNorm:
                 i / N and the 32-bit bit reversal of i over 2^32), N = 16
  mip_geometry   src/Render/Common/MipBuilder.h:142-181 (level k = previous // 2, stop at 0,
                 at most 10 levels) for every configured resolution
  deinterleave   bin/data/Shaders/glsl/Common/deinterleave.frag:16-28 and interleavedRendering.decl:2-7
                 (dst pixel p of the 4x4 grid reads src (p mod P) * G + p // P per axis), 8x8 image
  step_counts    indirectLighting.frag:167, 201-212 (n = int(ln(path / ns) / ln(2 pi / R + 1)) + 1,
                 ns = W / 1000, pi = 3.1415, path from BoxRayCast :83-99), in double precision

Run: python tests/golden/make_golden.py
"""
import json
import math
from pathlib import Path


def hammersley(i, n):
    b = int(format(i, "032b")[::-1], 2)
    return [i / n, b / 4294967296.0]


def mip_geometry(w, h, levels=10):
    sizes = [(w, h)]
    while len(sizes) < levels:
        nw, nh = sizes[-1][0] // 2, sizes[-1][1] // 2
        if nw == 0 or nh == 0:
            break
        sizes.append((nw, nh))
    return sizes


def deinterleave_source(w, h, g=4):
    pw, ph = w // g, h // g
    src = []
    for y in range(h):
        for x in range(w):
            sx = (x % pw) * g + x // pw
            sy = (y % ph) * g + y // ph
            src.append(sy * w + sx)
    return src


def step_count(w, h, r, cx, cy, dx, dy):
    pi = 3.1415
    ns = w / 1000.0
    tmax = []
    for (o, d, lim) in ((cx, dx, w), (cy, dy, h)):
        inv = 1.0 / d if d != 0 else math.copysign(math.inf, d)
        t1, t2 = (0 - o) * inv, (lim - o) * inv
        tmax.append(max(t1, t2))
    path = abs(min(tmax))
    return int(math.log(path / ns) / math.log(2 * pi / r + 1)) + 1


def main():
    res = [(1920, 1080), (512, 512), (640, 480), (256, 256), (1280, 720), (2048, 1152), (3840, 2160)]
    d = 1.0 / math.sqrt(1920 ** 2 + 1080 ** 2)
    kat = {
        "hammersley_16": [hammersley(i, 16) for i in range(16)],
        "mip_geometry": {f"{w}x{h}": mip_geometry(w, h) for w, h in res},
        "deinterleave_8x8_source": deinterleave_source(8, 8),
        "step_counts": [
            {"w": 1920, "h": 1080, "R": 4, "c": [960.5, 540.5], "d": [1.0, 0.0],
             "n": step_count(1920, 1080, 4, 960.5, 540.5, 1.0, 0.0)},
            {"w": 1920, "h": 1080, "R": 4, "c": [960.5, 540.5], "d": [0.0, 1.0],
             "n": step_count(1920, 1080, 4, 960.5, 540.5, 0.0, 1.0)},
            {"w": 1920, "h": 1080, "R": 4, "c": [0.5, 0.5], "d": [1920 * d, 1080 * d],
             "n": step_count(1920, 1080, 4, 0.5, 0.5, 1920 * d, 1080 * d)},
            {"w": 1920, "h": 1080, "R": 16, "c": [960.5, 540.5], "d": [1.0, 0.0],
             "n": step_count(1920, 1080, 16, 960.5, 540.5, 1.0, 0.0)},
            {"w": 512, "h": 512, "R": 8, "c": [256.5, 256.5], "d": [1.0, 0.0],
             "n": step_count(512, 512, 8, 256.5, 256.5, 1.0, 0.0)},
        ],
    }
    out = Path(__file__).with_name("kat.json")
    out.write_text(json.dumps(kat, indent=1))
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
