"""GPU tests of the learned reconstructor's pieces, through the C ABI: the
tile-list march, the feature builder, the BF16 tensor-core MLP (forward and
gradients against the FP64 oracle MLP), training, and checkpoints."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def dev(torch, a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    return t.cuda() if dtype is None else t.to(dtype).cuda()


def host(t):
    return t.detach().float().cpu().numpy()


@pytest.mark.parametrize("dirs,fast", [(8, False), (8, True), (24, True), (4, False)])
def test_march_tiles_equals_full_march(gi, cuda, scene_small, dirs, fast):
    """A tile list marches exactly the full march's values on its tiles.  With 8 to
    32 directions the list runs in the direction-split form (four threads per pixel,
    terms added in direction order), with fewer in the one-thread form."""
    torch = cuda
    s = scene_small
    gb, view = s["gb"], s["view"]
    W, H = view.width, view.height
    L = gi.mip_level_count(W, H, 10)
    ll, dl = gi.alloc_pyramid(W, H, 4, L), gi.alloc_pyramid(W, H, 2, L)
    ll[0].copy_(dev(torch, s["direct"]))
    dl[0].copy_(dev(torch, gb["moments"]))
    gi.build_mips(ll, 4)
    gi.build_mips(dl, 2)
    nrm, ndc = dev(torch, gb["normal"]), dev(torch, gb["ndc"])
    full = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    p = gi.GiMarchParams(dirs, 32, 4, 0, gi.GI_MARCH_FAST if fast else gi.GI_MARCH_EXACT)
    gi.march(view, p, ll, dl, nrm, ndc, full)
    tx, ty, tw, th = gi.march_tile_grid(W, H, 4)
    assert (tw, th) == (128, 16)
    tiles = torch.tensor([0, tx * ty - 1, tx + 1, 10_000, -3], dtype=torch.int32, device="cuda")  # two out of range
    part = torch.full((H, W, 4), -7.0, dtype=torch.float32, device="cuda")
    gi.march_tiles(view, p, ll, dl, nrm, ndc, part, tiles)
    f, g = host(full), host(part)
    mask = g[..., 3] != -7.0
    for t in (0, tx * ty - 1, tx + 1):
        x0, y0 = (t % tx) * tw, (t // tx) * th
        assert mask[y0:y0 + th, x0:x0 + tw].all()
    assert np.array_equal(f[mask], g[mask])
    assert mask.sum() == sum(min(tw, W - (t % tx) * tw) * min(th, H - (t // tx) * th)
                             for t in (0, tx * ty - 1, tx + 1))
    # gather / scatter round trip of the listed tiles
    gathered = torch.empty((3 * tw * th, 4), dtype=torch.float32, device="cuda")
    good = tiles[:3].contiguous()
    gi.gather_tiles(full, good, gathered)
    back = torch.zeros_like(full)
    gi.scatter_tiles(gathered, good, back)
    b = host(back)
    assert np.array_equal(b[mask], f[mask])


@pytest.mark.parametrize("fast", [False, True])
def test_march_tiles_edge_tiles(gi, cuda, fast):
    """Every tile of a 202x77 frame (partial tiles on the right and bottom, rows
    beyond the image inside the last tiles) marched as a tile list in the
    direction-split form equals the full march bit for bit."""
    torch = cuda
    from legitengine_gb300.train_reconstructor import Frame
    W, H = 202, 77
    fr = Frame(gi, torch, W, H)
    prims = gi.scene_generate(3001, 24, 4)
    pd, npr = gi.prims_to_device(prims)
    fr.inputs(pd, npr, gi.view_from_camera(gi.camera_spline(3001, 3, 64, prims), W, H),
              gi.view_from_camera(gi.scene_light(), 1024, 1024))
    p = gi.GiMarchParams(12, 32, 4, 0, gi.GI_MARCH_FAST if fast else gi.GI_MARCH_EXACT)
    full = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    gi.march(fr.view, p, fr.lb, fr.db, fr.normal, fr.ndc, full)
    tx, ty, tw, th = gi.march_tile_grid(W, H, 4)
    assert tx * tw > W and ty * th > H
    tiles = torch.arange(tx * ty, dtype=torch.int32, device="cuda").flip(0).contiguous()
    part = torch.full((H, W, 4), -7.0, dtype=torch.float32, device="cuda")
    gi.march_tiles(fr.view, p, fr.lb, fr.db, fr.normal, fr.ndc, part, tiles)
    assert np.array_equal(host(part), host(full))


def test_features_match_restatement(gi, cuda, scene_small):
    torch = cuda
    from oracle import mlp_oracle
    from oracle import oracle as O
    s = scene_small
    gb, view = s["gb"], s["view"]
    W, H = view.width, view.height
    rng = np.random.default_rng(3)
    ind0 = rng.uniform(0, 1, (H, W, 4)).astype(np.float32)
    i_l = O.mip_chain(ind0, 5)
    dblur = O.blur_pyramid(O.mip_chain(gb["moments"], 5))
    filt = rng.uniform(0, 1, (H, W, 4)).astype(np.float32)
    out = torch.empty((W * H, 32), dtype=torch.bfloat16, device="cuda")
    scale = torch.empty((W * H,), dtype=torch.float32, device="cuda")
    gi.features(dev(torch, gb["moments"]), dev(torch, gb["normal"]), dev(torch, gb["albedo"]),
                dev(torch, s["direct"]), [dev(torch, i_l[0]), dev(torch, i_l[2]), dev(torch, i_l[4])],
                dev(torch, filt), dev(torch, dblur[2]), out, scale)
    ys, xs = np.divmod(np.arange(W * H), W)
    ref, ref_scale = mlp_oracle.features(xs, ys, gb["moments"], gb["normal"], gb["albedo"], s["direct"], i_l[0],
                                         i_l[2], i_l[4], dblur[2], filtered=filt)
    assert np.allclose(host(scale), ref_scale, rtol=1e-6, atol=0)
    got = host(out)
    refb = mlp_oracle.bf16(ref)
    diff = np.abs(got - refb)
    assert np.mean(diff == 0) > 0.995
    assert np.all(diff <= np.abs(refb) * 2 ** -7 + 1e-6)
    # tile-list form: the same rows in tile-major order
    tx, ty, tw, th = gi.march_tile_grid(W, H, 4)
    tiles = torch.tensor([1, 2], dtype=torch.int32, device="cuda")
    outt = torch.empty((2 * tw * th, 32), dtype=torch.bfloat16, device="cuda")
    scalet = torch.empty((2 * tw * th,), dtype=torch.float32, device="cuda")
    gi.features(dev(torch, gb["moments"]), dev(torch, gb["normal"]), dev(torch, gb["albedo"]),
                dev(torch, s["direct"]), [dev(torch, i_l[0]), dev(torch, i_l[2]), dev(torch, i_l[4])],
                dev(torch, filt), dev(torch, dblur[2]), outt, scalet, tiles=tiles)
    gt = host(outt).reshape(2, th, tw, 32)
    full = got.reshape(H, W, 32)
    for k, t in enumerate((1, 2)):
        x0, y0 = (t % tx) * tw, (t // tx) * th
        hh, ww = min(th, H - y0), min(tw, W - x0)
        assert np.array_equal(gt[k, :hh, :ww], full[y0:y0 + hh, x0:x0 + ww])


def _batch(rng, n):
    x = rng.normal(0, 1, (n, 32)).astype(np.float32)
    t = np.zeros((n, 4), np.float32)
    t[:, :3] = rng.uniform(0, 1, (n, 3))
    t[:, 3] = rng.uniform(0.25, 2.0, n)  # per-pixel loss weight
    return x, t


def test_mlp_forward_matches_fp64_oracle(gi, cuda):
    torch = cuda
    from oracle import mlp_oracle as M
    net = gi.Mlp(seed=11)
    p = M.unpack(net.get_params())
    x, _ = _batch(np.random.default_rng(1), 1000)  # not a multiple of the 64-pixel tile
    out = torch.empty((1000, 4), dtype=torch.float32, device="cuda")
    net.forward(dev(torch, x, torch.bfloat16), out)
    y, _ = M.forward(p, x)
    got = host(out)
    assert np.all(got[:, 3] == 1.0)
    assert np.abs(y).max() > 0
    err = np.abs(got[:, :3] - y).max() / np.abs(y).max()
    print(f"mlp forward max err {err:.3g}")
    assert err < 1e-2


def test_mlp_exposure_scale(gi, cuda):
    """Forward multiplies by the scale; training divides targets by it."""
    torch = cuda
    from oracle import mlp_oracle as M
    net = gi.Mlp(seed=12)
    x, t = _batch(np.random.default_rng(6), 640)
    sc = np.random.default_rng(8).uniform(0.01, 3.0, 640).astype(np.float32)
    xd = dev(torch, x, torch.bfloat16)
    a = torch.empty((640, 4), dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    net.forward(xd, a)
    net.forward(xd, b, scale=dev(torch, sc))
    assert torch.allclose(b[:, :3], a[:, :3] * dev(torch, sc)[:, None], rtol=1e-6, atol=0)
    l1, g1 = net.gradients(xd, dev(torch, t), scale=dev(torch, sc))
    ts = t.copy()
    ts[:, :3] /= sc[:, None]
    l2, g2 = net.gradients(xd, dev(torch, ts))
    assert abs(l1 - l2) <= 1e-5 * l2
    assert np.allclose(g1, g2, rtol=1e-3, atol=1e-6)


GRAD_RTOL = 5e-3  # relative L2 error per tensor against the bf16-rounded oracle


@pytest.mark.parametrize("n,loss", [(77, "squared"), (4096, "squared"), (100_003, "squared"), (4096, "absolute"),
                                    (100_003, "absolute")])
def test_mlp_gradients_match_fp64_oracle(gi, cuda, n, loss):
    """The tensor-core training kernel's loss and gradients against the FP64
    oracle that rounds to bf16 where the kernel does (inputs, weights, hidden
    activations, the logits' gradient, the masked hidden gradients): each
    tensor within GRAD_RTOL relative L2.  n = 77 is one partial tile; 4096 is
    one tile per CTA; 100 003 gives each CTA several tiles (the weight
    gradients accumulate in tensor memory across them) and a ragged last tile.
    Both training losses: the clipped squared error (the default) and the
    absolute error (GI_MLP_LOSS_ABSOLUTE)."""
    torch = cuda
    from oracle import mlp_oracle as M
    net = gi.Mlp(seed=5)
    if loss == "absolute":
        net.set_loss(gi.GI_MLP_LOSS_ABSOLUTE)
    p = M.unpack(net.get_params())
    x, t = _batch(np.random.default_rng(2 + n), n)
    lv, g = net.gradients(dev(torch, x, torch.bfloat16), dev(torch, t))
    lref, gref = M.loss_and_grad(p, x, t, loss=loss)
    _, g64 = M.loss_and_grad(p, x, t, use_bf16=False, loss=loss)
    assert abs(lv - lref) / lref < 1e-4
    gg = M.unpack(g)
    for name, _ in M.SHAPES:
        e = np.linalg.norm(gg[name] - gref[name]) / np.linalg.norm(gref[name])
        e64 = np.linalg.norm(gg[name] - g64[name]) / np.linalg.norm(g64[name])
        print(f"n={n} {loss} grad {name}: rel err vs bf16-rounded oracle {e:.2e}, vs pure fp64 {e64:.2e}")
        assert e < GRAD_RTOL, name
        assert e64 < 1e-1, name


def test_mlp_training_fits_a_teacher(gi, cuda):
    """Adam on a fixed regression (a random teacher network): the loss falls by 10x."""
    torch = cuda
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(7)
    teacher = M.unpack(rng.normal(0, 0.3, M.PARAMS))
    x = rng.normal(0, 1, (16384, 32)).astype(np.float32)
    y, _ = M.forward(teacher, x, use_bf16=False)
    t = np.ones((16384, 4), np.float32)
    t[:, :3] = y
    net = gi.Mlp(seed=3)
    xd, td = dev(torch, x, torch.bfloat16), dev(torch, t)
    first = net.train_step(xd, td, lr=2e-3)
    for _ in range(600):
        last = net.train_step(xd, td, lr=2e-3, want_loss=False)
    last = net.train_step(xd, td, lr=2e-3)
    print(f"teacher fit: loss {first:.4g} -> {last:.4g}")
    assert last < 0.1 * first


def test_mlp_loss_selection(gi, cuda):
    """gi_mlp_set_loss takes the two losses and refuses anything else, and it is
    the training step's: the gradients differ between the two on the same batch
    and come back (to the order of the CTAs' atomic additions) when the loss is
    set back."""
    torch = cuda
    net = gi.Mlp(seed=21)
    x, t = _batch(np.random.default_rng(21), 512)
    xd, td = dev(torch, x, torch.bfloat16), dev(torch, t)
    _, g_sq = net.gradients(xd, td)
    net.set_loss(gi.GI_MLP_LOSS_ABSOLUTE)
    _, g_abs = net.gradients(xd, td)
    net.set_loss(gi.GI_MLP_LOSS_SQUARED)
    _, g_sq2 = net.gradients(xd, td)
    scale = np.abs(g_sq).max()
    assert np.abs(g_sq - g_sq2).max() <= 1e-5 * scale
    assert np.abs(g_sq - g_abs).max() > 1e-2 * scale
    for bad in (-1, 2, 7):
        with pytest.raises(gi.GiError) as e:
            net.set_loss(bad)
        assert e.value.status == gi.GI_ERR_INVALID_ARGUMENT


def test_mlp_checkpoint_round_trip(gi, cuda, tmp_path):
    torch = cuda
    net = gi.Mlp(seed=9)
    x, t = _batch(np.random.default_rng(4), 512)
    xd, td = dev(torch, x, torch.bfloat16), dev(torch, t)
    for _ in range(3):
        net.train_step(xd, td, lr=1e-3, want_loss=False)
    path = tmp_path / "net.bin"
    net.save(path)
    other = gi.Mlp(seed=None)
    other.load(path)
    assert np.array_equal(net.get_params(), other.get_params())
    a = torch.empty((512, 4), dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    net.forward(xd, a)
    other.forward(xd, b)
    assert torch.equal(a, b)
    # Adam state travels too: one more step on the same batch moves both alike (gradient partials are
    # summed with atomics, so the last bits may differ).
    before = net.get_params()
    net.train_step(xd, td, want_loss=False)
    other.train_step(xd, td, want_loss=False)
    a, b = net.get_params(), other.get_params()
    assert np.abs(a - b).max() <= 1e-4 * np.abs(a - before).max()
    raw = bytearray(path.read_bytes())
    raw[100] ^= 0x40
    path.write_bytes(bytes(raw))
    with pytest.raises(gi.GiError) as ei:
        other.load(path)
    assert ei.value.status == 6 and "CRC" in str(ei.value)


def test_renderer_learned_mode_and_judge(gi, cuda):
    """Learned mode end to end at 320x240 (1 bounce).  With threshold 0 every judged tile falls
    back, so those tiles carry exactly the plain march; the other tiles carry the network's output."""
    torch = cuda
    W, H = 320, 240
    prims = gi.scene_generate(4001, 64, 16)
    pd, npr = gi.prims_to_device(prims)
    view = gi.view_from_camera(gi.camera_spline(7, 3, 64, prims), W, H)
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    f = dict(dtype=torch.float32, device="cuda")
    t = {k: torch.empty((H, W, c), **f) for k, c in (("albedo", 4), ("emissive", 4), ("normal", 4),
                                                     ("moments", 2), ("ndc", 1), ("direct", 4))}
    sm = torch.empty((512, 512, 1), **f)
    gi.gbuffer(view, pd, npr, t["albedo"], t["emissive"], t["normal"], t["moments"], t["ndc"])
    gi.shadow_map(light, pd, npr, sm)
    gi.direct_light(view, light, t["albedo"], t["emissive"], t["normal"], t["ndc"], sm, t["direct"])
    net = gi.Mlp(seed=2)
    r = gi.Renderer(W, H, dirs=8, step_cap=32, bounces=1)
    r.set_learned(net, few_dirs=2, few_step_dirs=16, judge_every=4, threshold=0.0)
    lit, ind = torch.empty((H, W, 4), **f), torch.empty((H, W, 4), **f)
    r.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit, ind)
    torch.cuda.synchronize()
    judged, fell = r.stats()
    tx, ty, tw, th = gi.march_tile_grid(W, H, 4)
    assert judged == len(range(0, tx * ty, 4)) and fell == judged
    # the plain march of the same frame
    L = gi.mip_level_count(W, H, 10)
    ll, dl = [t["direct"]] + gi.alloc_pyramid(W, H, 4, L)[1:], [t["moments"]] + gi.alloc_pyramid(W, H, 2, L)[1:]
    gi.build_mips(ll, 4)
    gi.build_mips(dl, 2)
    lb, db = [ll[0]] + gi.alloc_pyramid(W, H, 4, L)[1:], [dl[0]] + gi.alloc_pyramid(W, H, 2, L)[1:]
    gi.blur_pyramid(ll, lb)
    gi.blur_pyramid(dl, db)
    plain = torch.empty((H, W, 4), **f)
    gi.march(view, gi.GiMarchParams(8, 32, 4), lb, db, t["normal"], t["ndc"], plain)
    torch.cuda.synchronize()
    a, p = ind.cpu().numpy(), plain.cpu().numpy()
    assert np.isfinite(a).all()
    for tile in range(0, tx * ty, 4):
        x0, y0 = (tile % tx) * tw, (tile // tx) * th
        assert np.array_equal(a[y0:y0 + th, x0:x0 + tw], p[y0:y0 + th, x0:x0 + tw])
    # a tile that was not judged holds the network's (different) result
    x0, y0 = (1 % tx) * tw, (1 // tx) * th
    assert not np.array_equal(a[y0:y0 + th, x0:x0 + tw], p[y0:y0 + th, x0:x0 + tw])
    # back to the plain method
    r.set_learned(None)
    r.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit, ind)
    torch.cuda.synchronize()


def _reconstruct_inputs(torch, W, H, rng):
    """Random but plausible inputs of the feature builder at W x H."""
    from oracle import oracle as O
    d = rng.uniform(0.5, 3.0, (H, W)).astype(np.float32)
    mom = np.stack([d, d * d * rng.uniform(1.0, 1.05, (H, W)).astype(np.float32)], -1).astype(np.float32)
    nrm = np.concatenate([rng.normal(0, 1, (H, W, 3)), np.ones((H, W, 1))], -1).astype(np.float32)
    alb = rng.uniform(0.2, 0.9, (H, W, 4)).astype(np.float32)
    dl = rng.uniform(0, 2, (H, W, 4)).astype(np.float32)
    ind0 = rng.uniform(0, 1, (H, W, 4)).astype(np.float32)
    i_l = O.mip_chain(ind0, 5)
    dblur = O.blur_pyramid(O.mip_chain(mom, 5))
    filt = rng.uniform(0, 1, (H, W, 4)).astype(np.float32)
    t = {"moments": dev(torch, mom), "normal": dev(torch, nrm), "albedo": dev(torch, alb), "direct": dev(torch, dl),
         "levels": [dev(torch, i_l[0]), dev(torch, i_l[2]), dev(torch, i_l[4])], "filtered": dev(torch, filt),
         "dl2": dev(torch, dblur[2])}
    return t


@pytest.mark.parametrize("size", [(128, 96), (650, 363)])
def test_reconstruct_tensor_cores_matches_features_and_forward(gi, cuda, size):
    """The fused tcgen05 kernel against gi_features + gi_mlp_forward (the same
    tensor-core network on the feature rows gi_features writes: equal bits) and
    against the FP64 oracle network on the same bf16 features.  650 x 363 has
    more tiles than the persistent grid (CTAs loop) and ends on a partial
    128-pixel tile."""
    torch = cuda
    from oracle import mlp_oracle as M
    W, H = size
    t = _reconstruct_inputs(torch, W, H, np.random.default_rng(W))
    net = gi.Mlp(seed=W)
    before = gi.tensor_core_errors()
    fused = torch.full((H, W, 4), -1.0, dtype=torch.float32, device="cuda")
    net.reconstruct(t["moments"], t["normal"], t["albedo"], t["direct"], t["levels"], t["filtered"], t["dl2"], fused)
    X = torch.empty((W * H, 32), dtype=torch.bfloat16, device="cuda")
    S = torch.empty((W * H,), dtype=torch.float32, device="cuda")
    gi.features(t["moments"], t["normal"], t["albedo"], t["direct"], t["levels"], t["filtered"], t["dl2"], X, S)
    ref = torch.empty((W * H, 4), dtype=torch.float32, device="cuda")
    net.forward(X, ref, scale=S)
    torch.cuda.synchronize()
    assert gi.tensor_core_errors() == before
    got = host(fused).reshape(-1, 4)
    assert np.all(got[:, 3] == 1.0)
    r = host(ref)
    y, _ = M.forward(M.unpack(net.get_params()), host(X))
    y = y * host(S)[:, None]
    mag = np.abs(y).max()
    e_ref = np.abs(got[:, :3] - r[:, :3]).max() / mag
    e_o = np.abs(got[:, :3] - y).max() / mag
    e_mean = np.abs(got[:, :3] - y).mean() / np.abs(y).mean()
    same = float(np.mean(got == r))
    print(f"fused vs features + forward: max {e_ref:.3g}, bit-identical {same * 100:.3f}%; "
          f"vs fp64 max {e_o:.3g} mean {e_mean:.3g}")
    assert np.isfinite(got).all()
    assert same >= 0.999 and e_ref < 1e-5
    assert e_o < 1e-2 and e_mean < 1e-3
    # the hidden layers are live: the blend is not the uniform one
    xb = M.bf16(host(X))
    uniform = (xb[:, 10:13] + xb[:, 19:22] + xb[:, 22:25]) / 3 * host(S)[:, None]
    assert np.abs(y - uniform).mean() > 0.01 * np.abs(y).mean()


def test_learned_network_gain_over_its_candidates(gi, cuda):
    """What the trained network gains over the method without it, on the bench's
    4 held-out 1920x1080 frames (scene seeds 20000-20003, never trained on): its
    relative L1 error against the bilaterally filtered R = 256 gather, next to each
    candidate estimate it blends taken alone -- the few-ray light after the 5x5
    bilateral, and its mip-2 (4x4 box, bilinear) average -- and to the plain
    R = 16 gather.  The network must beat the bilateral candidate and the plain
    R = 16 gather by far and be no worse than its best candidate (mip 2)."""
    from legitengine_gb300 import train_reconstructor as tr
    net = gi.Mlp(seed=None)
    net.load(tr.DEFAULT_WEIGHTS)
    ev = tr.evaluate(net, frames=4, few_dirs=tr.DEFAULT_FEW_DIRS, few_step_dirs=tr.DEFAULT_FEW_STEP_DIRS,
                     plain_dirs=(16,), precision=gi.GI_MARCH_TEXTURE, verbose=False)
    learned, mip2, few, plain = (ev[k]["error"] for k in ("learned", "few_mip2", "few", "plain16"))
    print(f"held-out error: learned {learned:.4f}, mip-2 candidate {mip2:.4f} (gain {mip2 / learned:.3f}), "
          f"bilateral candidate {few:.4f} (gain {few / learned:.2f}), plain R=16 {plain:.4f} "
          f"(gain {plain / learned:.2f})")
    assert learned < 0.5 * few
    assert learned < 0.85 * plain
    assert learned <= mip2 * 1.0001
