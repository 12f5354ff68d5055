"""Writes tests/golden/texture_unit_weights.npz: texel weights of the GPU's
texture units, measured through the library's own texture path
(legitengine_gb300.gi.texture_sample, the fetch GI_MARCH_TEXTURE takes).

Method: a 256x64 pyramid of 4 levels; pyramid (l, p) is 1 on the texels of
level l whose (x % 2, y % 2) is parity class p = (x % 2) + 2 (y % 2), and 0
elsewhere.  A bilinear footprint holds one texel of each parity class, so a
fetch from pyramid (l, p) returns the weight of that footprint texel at level l.
3000 random points (coordinates in [0.05, 0.95]^2, levels in [0, 3)) against all
16 pyramids give the eight trilinear weights of every point.  Stored: the points
(float32) and the weights times 256 (uint16: every weight is a multiple of 1/256).

Run on a machine with the GPU:  python tests/golden/make_texture_weights.py [OUT]
"""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[2]))

W, H, L, N = 256, 64, 4, 3000


def main(out: Path):
    import torch
    from legitengine_gb300 import gi
    rng = np.random.default_rng(2026)
    coords = np.stack([rng.uniform(0.05, 0.95, N), rng.uniform(0.05, 0.95, N)], -1).astype(np.float32)
    lods = rng.uniform(0.0, 3.0, N).astype(np.float32)
    dc = torch.from_numpy(coords).cuda()
    dl = torch.from_numpy(lods).cuda()
    weights = np.zeros((L, 4, N), np.uint16)
    for lev in range(L):
        for p in range(4):
            levels = []
            for k in range(L):
                w, h = W >> k, H >> k
                a = np.zeros((h, w, 1), np.float32)
                if k == lev:
                    a[(p >> 1)::2, (p & 1)::2, 0] = 1.0
                levels.append(torch.from_numpy(a).cuda())
            got = torch.empty((N, 1), dtype=torch.float32, device="cuda")
            gi.texture_sample(levels, 1, dc, dl, got)
            torch.cuda.synchronize()
            g = got.cpu().numpy()[:, 0] * 256.0
            assert np.all(np.abs(g - np.rint(g)) < 1e-4), "a weight off the 1/256 grid"
            weights[lev, p] = np.rint(g).astype(np.uint16)
    np.savez_compressed(out, coords=coords, lods=lods, weights=weights, size=np.array([W, H, L]))
    print("wrote", out)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).parent / "texture_unit_weights.npz")
