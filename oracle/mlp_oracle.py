"""FP64 restatement of the learned reconstructor (TEST INFRASTRUCTURE ONLY).

Forward and backward of the 32 -> 64 -> 64 -> 64 -> 3 ReLU MLP, its softmax
output head (the 3 outputs weight a blend of three candidate estimates held in
the input row: channels 10-12, 19-21 and 22-24) and the weighted squared error,
written from the mathematics.  With bf16=True the values the
CUDA kernels round to bf16 (inputs, weights, hidden activations, the output
error and the masked hidden errors) are rounded the same way (round to
nearest even), everything else is float64.
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT = 32, 64, 3
CANDIDATES = (10, 19, 22)  # first channel of each candidate estimate blended by the head
SHAPES = [("W1", (IN, HID)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)), ("W3", (HID, HID)),
          ("b3", (HID,)), ("W4", (HID, OUT)), ("b4", (OUT,))]
PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(flat: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(flat[o:o + n], np.float64).reshape(shape)
        o += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([d[name].ravel() for name, _ in SHAPES])


def forward(p: dict, x: np.ndarray, use_bf16=True):
    r = bf16 if use_bf16 else (lambda a: np.asarray(a, np.float64))
    W = {k: (r(v) if k.startswith("W") else v) for k, v in p.items()}
    x = r(x)
    h1 = r(np.maximum(x @ W["W1"] + p["b1"], 0))
    h2 = r(np.maximum(h1 @ W["W2"] + p["b2"], 0))
    h3 = r(np.maximum(h2 @ W["W3"] + p["b3"], 0))
    o = h3 @ W["W4"] + p["b4"]
    c = np.stack([x[:, k:k + OUT] for k in CANDIDATES], 1)  # [n, 3 candidates, 3 channels]
    e = np.exp(o - o.max(1, keepdims=True))
    w = e / e.sum(1, keepdims=True)
    y = (w[:, :, None] * c).sum(1)
    return y, (x, h1, h2, h3, W, w, c)


def loss_and_grad(p: dict, x: np.ndarray, t: np.ndarray, use_bf16=True, loss="squared"):
    """Weighted mean loss over the batch and the 3 outputs (t: [n, 3], or [n, 4]
    with the pixel's loss weight in column 3) and its gradient, as in the kernels
    (gi_mlp_layout.h head_loss_grad_logits): loss="squared", w e^2 with the
    per-output error clipped to [-1, 1] in the gradient; loss="absolute", w |e|
    with gradient w sign(e)."""
    r = bf16 if use_bf16 else (lambda a: np.asarray(a, np.float64))
    y, (x, h1, h2, h3, W, sw, c) = forward(p, x, use_bf16)
    n = x.shape[0]
    w = t[:, 3:4].astype(np.float64) if t.shape[1] > OUT else np.ones((n, 1))
    e = y - t[:, :OUT]
    if loss == "absolute":
        lossv = float((w * np.abs(e)).sum() / (n * OUT))
        g = w * np.sign(e)  # gradient of the summed loss at y
    else:
        lossv = float((w * e ** 2).sum() / (n * OUT))
        g = 2.0 * w * np.clip(e, -1.0, 1.0)  # gradient of the summed loss at y, error clipped to [-1, 1]
    dy = r(sw * (g[:, None, :] * (c - y[:, None, :])).sum(2))  # through the softmax blend, at the logits
    g = {"W4": h3.T @ dy, "b4": dy.sum(0)}
    dz3 = r((dy @ W["W4"].T) * (h3 > 0))
    g.update({"W3": h2.T @ dz3, "b3": dz3.sum(0)})
    dz2 = r((dz3 @ W["W3"].T) * (h2 > 0))
    g.update({"W2": h1.T @ dz2, "b2": dz2.sum(0)})
    dz1 = r((dz2 @ W["W2"].T) * (h1 > 0))
    g.update({"W1": x.T @ dz1, "b1": dz1.sum(0)})
    return lossv, {k: v / n for k, v in g.items()}


def _bilinear(img: np.ndarray, s: np.ndarray, t: np.ndarray) -> np.ndarray:
    """Vulkan linear filter, clamp-to-edge, fp32 arithmetic in the library's order
    (weights summed t00, t10, t01, t11; division as a * (1 / b))."""
    h, w = img.shape[:2]
    f32 = np.float32

    def setup(c, n):
        u = (c.astype(f32) * f32(n)).astype(f32)
        uu = (u - f32(0.5)).astype(f32)
        fl = np.floor(uu).astype(f32)
        a = (uu - fl).astype(f32)
        i = np.clip(fl, -1e6, 1e6).astype(np.int64)
        return np.clip(i, 0, n - 1), np.clip(i + 1, 0, n - 1), a

    i0, i1, a = setup(s, w)
    j0, j1, b = setup(t, h)
    oa, ob = (f32(1) - a).astype(f32), (f32(1) - b).astype(f32)
    w00, w10, w01, w11 = (oa * ob).astype(f32), (a * ob).astype(f32), (oa * b).astype(f32), (a * b).astype(f32)
    r = img[j0, i0] * w00[:, None]
    r = (r + img[j0, i1] * w10[:, None]).astype(f32)
    r = (r + img[j1, i0] * w01[:, None]).astype(f32)
    r = (r + img[j1, i1] * w11[:, None]).astype(f32)
    return r


FEATURE_LIMIT = 32.0  # normalised light features are clamped to [-32, 32]


def features(xs, ys, moments, normal, albedo, direct, ind0, ind2, ind4, depth_l2, pattern=4, filtered=None):
    """The 32 features of pixels (xs, ys), float32 before the bf16 rounding (channel
    layout of the CUDA feature builder), and the exposure scale the light-dependent
    channels were divided by."""
    f32 = np.float32
    H, W = normal.shape[:2]
    n = len(xs)
    F = np.zeros((n, 32), f32)
    F[:, 0] = moments[ys, xs, 0]
    F[:, 1:4] = normal[ys, xs, :3]
    F[:, 4:7] = albedo[ys, xs, :3]
    F[:, 7:10] = ind0[ys, xs, :3]
    F[:, 10:13] = filtered[ys, xs, :3]
    for k, (dx, dy) in enumerate(((-1, 0), (1, 0), (0, -1), (0, 1), (-1, -1), (1, 1))):
        c = ind0[np.clip(ys + dy, 0, H - 1), np.clip(xs + dx, 0, W - 1)]
        F[:, 13 + k] = (f32(0.2126) * c[:, 0] + f32(0.7152) * c[:, 1] + f32(0.0722) * c[:, 2]).astype(f32)
    s = ((xs.astype(f32) + f32(0.5)) / f32(W)).astype(f32)
    t = ((ys.astype(f32) + f32(0.5)) / f32(H)).astype(f32)
    F[:, 19:22] = _bilinear(ind2, s, t)[:, :3]
    F[:, 22:25] = _bilinear(ind4, s, t)[:, :3]
    m = depth_l2[np.clip(ys >> 2, 0, depth_l2.shape[0] - 1), np.clip(xs >> 2, 0, depth_l2.shape[1] - 1)]
    F[:, 25] = np.sqrt(np.maximum(0, m[:, 1] - m[:, 0] * m[:, 0]))
    F[:, 26:29] = direct[ys, xs, :3]
    pidx = (xs % pattern) + (ys % pattern) * pattern
    F[:, 29] = pidx / f32(pattern * pattern)
    F[:, 30] = [int(format(int(i), "032b")[::-1], 2) * 2.3283064365386963e-10 for i in pidx]
    F[:, 31] = np.minimum(np.minimum(s, 1 - s), np.minimum(t, 1 - t))
    lum = lambda c: (f32(0.2126) * c[:, 0] + f32(0.7152) * c[:, 1] + f32(0.0722) * c[:, 2]).astype(f32)
    i2 = _bilinear(ind2, s, t)
    i4 = _bilinear(ind4, s, t)
    scale = ((np.abs(lum(i2)) + np.abs(lum(i4))).astype(f32) + f32(1e-3)).astype(f32)
    rs = (f32(1) / scale).astype(f32)
    lim = f32(FEATURE_LIMIT)
    F[:, 7:25] = np.clip((F[:, 7:25] * rs[:, None]).astype(f32), -lim, lim)
    F[:, 26:29] = np.clip((F[:, 26:29] * rs[:, None]).astype(f32), -lim, lim)
    return F, scale
