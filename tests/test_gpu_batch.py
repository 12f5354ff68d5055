"""Batched views (one persistent march launch for many views of uneven size,
replayed as a CUDA graph) and the march autotuner, through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(gi, torch, seed, W, H, light):
    prims = gi.scene_generate(seed, 16 + seed % 48, seed % 8)
    pd, npr = gi.prims_to_device(prims)
    view = gi.view_from_camera(gi.camera_spline(seed, seed % 64, 64, prims), W, H)
    f = dict(dtype=torch.float32, device="cuda")
    t = {k: torch.empty((H, W, c), **f) for k, c in (("albedo", 4), ("emissive", 4), ("normal", 4),
                                                     ("moments", 2), ("ndc", 1), ("direct", 4))}
    sm = torch.empty((512, 512, 1), **f)
    gi.gbuffer(view, pd, npr, t["albedo"], t["emissive"], t["normal"], t["moments"], t["ndc"])
    gi.shadow_map(light, pd, npr, sm)
    gi.direct_light(view, light, t["albedo"], t["emissive"], t["normal"], t["ndc"], sm, t["direct"])
    return view, t


VIEWS = [(160, 128, 8, 0, 32, 0), (256, 256, 16, 0, 64, 1), (320, 240, 4, 0, 0, 0), (128, 96, 12, 0, 16, 2),
         (210, 118, 2, 32, 64, 1), (64, 64, 24, 0, 64, 0), (176, 100, 16, 0, 64, 2)]
# W, H, R, step_dirs, cap, precision (0 exact, 1 fast, 2 texture)


@pytest.mark.parametrize("tile_rows", [0, 2])
def test_batch_matches_single_view_renderer(gi, cuda, tile_rows):
    torch = cuda
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    specs = []
    for k, (W, H, R, SR, cap, prec) in enumerate(VIEWS):
        view, t = _inputs(gi, torch, 300 + k, W, H, light)
        t["out_lit"] = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        t["out_indirect"] = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        specs.append(dict(view=view, march=gi.GiMarchParams(R, cap, 4, SR, prec), **t))
    torch.cuda.synchronize()
    b = gi.Batch(specs, tile_rows=tile_rows)
    info = b.info()
    assert info["tile_rows"] in (2, 4, 8) and info["work_items"] > 0 and info["grid"] > 0
    if tile_rows:
        assert info["tile_rows"] == tile_rows
    stream = torch.cuda.Stream()
    import ctypes as C
    b.render(C.c_void_p(stream.cuda_stream))
    stream.synchronize()
    first = [(s["out_lit"].clone(), s["out_indirect"].clone()) for s in specs]
    b.render(C.c_void_p(stream.cuda_stream))  # graph replay
    stream.synchronize()
    for s, (l0, i0) in zip(specs, first):
        assert torch.equal(s["out_lit"], l0) and torch.equal(s["out_indirect"], i0)
    for s, (W, H, R, SR, cap, prec) in zip(specs, VIEWS):
        r = gi.Renderer(W, H, dirs=R, step_cap=cap, bounces=1, bilateral=True, step_dirs=SR, precision=prec)
        lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        ind = torch.empty_like(lit)
        r.render(s["view"], s["albedo"], s["normal"], s["moments"], s["ndc"], s["direct"], lit, ind)
        torch.cuda.synchronize()
        r.close()
        assert torch.equal(ind, s["out_indirect"]), (W, H, R)
        assert torch.equal(lit, s["out_lit"]), (W, H, R)


def test_batch_of_more_views_than_one_launch_holds(gi, cuda):
    """53 views of one precision: more than the 48 views one persistent launch
    takes as its parameter, so the work list runs in two launches; every view's
    image equals the single-view renderer's bit for bit."""
    torch = cuda
    import ctypes as C
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    rng = np.random.default_rng(53)
    specs, shapes = [], []
    for k in range(53):
        W, H, R = int(rng.integers(40, 97)), int(rng.integers(24, 65)), int(rng.integers(2, 13))
        view, t = _inputs(gi, torch, 700 + k, W, H, light)
        t["out_lit"] = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        specs.append(dict(view=view, march=gi.GiMarchParams(R, 24, 4, 0, 1), **t))
        shapes.append((W, H, R))
    torch.cuda.synchronize()
    b = gi.Batch(specs, tile_rows=4)
    stream = torch.cuda.Stream()
    b.render(C.c_void_p(stream.cuda_stream))
    stream.synchronize()
    for s, (W, H, R) in zip(specs, shapes):
        r = gi.Renderer(W, H, dirs=R, step_cap=24, bounces=1, bilateral=True, precision=1)
        lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        r.render(s["view"], s["albedo"], s["normal"], s["moments"], s["ndc"], s["direct"], lit)
        torch.cuda.synchronize()
        r.close()
        assert torch.equal(lit, s["out_lit"]), (W, H, R)
    b.close()


def _march_inputs(gi, torch, W, H):
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    view, t = _inputs(gi, torch, 77, W, H, light)
    L = gi.mip_level_count(W, H, 10)
    lb = [t["direct"]] + gi.alloc_pyramid(W, H, 4, L)[1:]
    db = [t["moments"]] + gi.alloc_pyramid(W, H, 2, L)[1:]
    ll = [t["direct"]] + gi.alloc_pyramid(W, H, 4, L)[1:]
    dl = [t["moments"]] + gi.alloc_pyramid(W, H, 2, L)[1:]
    gi.build_mips(ll, 4)
    gi.build_mips(dl, 2)
    gi.blur_pyramid(ll, lb)
    gi.blur_pyramid(dl, db)
    return view, t, lb, db


@pytest.mark.parametrize("dirs,precision", [(12, 0), (12, 2), (2, 1)])
def test_autotuner_records_a_shape_and_keeps_results(gi, cuda, dirs, precision):
    """The autotuner times CTA heights 2, 4, 8 (one thread per pixel: 32 x dirs
    rays per warp) and, for 4 to 32 directions, the direction split (32 x
    ceil(dirs / 4)); it records its choice for the shape, and tuned output
    equals untuned bit for bit."""
    torch = cuda
    W, H = 640, 360
    view, t, lb, db = _march_inputs(gi, torch, W, H)
    p = gi.GiMarchParams(dirs, 40, 4, 0, precision)
    base = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    gi.march(view, p, lb, db, t["normal"], t["ndc"], base)  # untuned: the default layout
    assert gi.march_tuned_layout(W, H, dirs, 0, 40, precision) == (0, 0)
    out = torch.empty_like(base)
    rows, rpw, ms = gi.march_autotune(view, p, lb, db, t["normal"], t["ndc"], out)
    print(f"{W}x{H} R={dirs} precision {precision}: {rows} rows, {rpw} rays per warp, {ms:.3f} ms")
    allowed = {(2, 32 * dirs), (4, 32 * dirs), (8, 32 * dirs)}
    if 4 <= dirs <= 32:
        allowed.add((4, 32 * ((dirs + 3) // 4)))
    assert (rows, rpw) in allowed and ms > 0
    assert gi.march_tuned_layout(W, H, dirs, 0, 40, precision) == (rows, rpw)
    if precision == 0:
        assert gi.lib().gi_march_tuned_rows(W, H, dirs, 0, 40) == rows
    tuned = torch.empty_like(base)
    gi.march(view, p, lb, db, t["normal"], t["ndc"], tuned)
    torch.cuda.synchronize()
    assert torch.equal(tuned, base) and torch.equal(out, base)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_every_march_layout_gives_the_same_frame(gi, cuda, precision):
    """Each layout pinned with gi_march_set_layout -- 2, 4, 8 rows and the
    direction split -- on a frame whose size is no multiple of the tiles, and
    with 5, 12 and 32 directions: bit-identical frames.  Layouts the shape
    cannot take are refused."""
    torch = cuda
    W, H = 333, 207
    view, t, lb, db = _march_inputs(gi, torch, W, H)
    for dirs in (5, 12, 32):
        p = gi.GiMarchParams(dirs, 48, 4, 0, precision)
        frames = []
        for rows, rpw in ((2, 32 * dirs), (4, 32 * dirs), (8, 32 * dirs), (4, 32 * ((dirs + 3) // 4))):
            gi.march_set_layout(W, H, dirs, 0, 48, precision, rows, rpw)
            assert gi.march_tuned_layout(W, H, dirs, 0, 48, precision) == (rows, rpw)
            o = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
            gi.march(view, p, lb, db, t["normal"], t["ndc"], o)
            frames.append(o)
        torch.cuda.synchronize()
        for o in frames[1:]:
            assert torch.equal(o, frames[0]), dirs
    for bad in ((3, 32 * 12), (2, 32 * 3), (4, 100)):
        with pytest.raises(gi.GiError):
            gi.march_set_layout(W, H, 12, 0, 48, precision, *bad)
    with pytest.raises(gi.GiError):  # 2 directions: no split
        gi.march_set_layout(W, H, 2, 0, 48, precision, 4, 32)


@pytest.mark.parametrize("precision", [0, 2])
def test_renderer_frame_is_the_same_in_every_layout(gi, cuda, precision):
    """The two-bounce renderer (bounce 1 records its march, bounce 2 replays it)
    under each pinned layout of its march shape: the recording march and the
    replay take the layout's CTA rows and ignore the direction split (a record
    is written one thread per pixel); the lit image is the same bits in all."""
    torch = cuda
    W, H, R, cap = 301, 187, 12, 40
    view, t, _, _ = _march_inputs(gi, torch, W, H)
    frames = []
    for rows, rpw in ((4, 32 * R), (2, 32 * R), (8, 32 * R), (4, 32 * ((R + 3) // 4))):
        gi.march_set_layout(W, H, R, 0, cap, precision, rows, rpw)
        r = gi.Renderer(W, H, dirs=R, step_cap=cap, bounces=2, bilateral=True, precision=precision)
        lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        r.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], t["direct"], lit)
        torch.cuda.synchronize()
        r.close()
        frames.append(lit)
    for lit in frames[1:]:
        assert torch.equal(lit, frames[0])


def test_learned_batch_matches_learned_renderer_and_finetunes(gi, cuda):
    """Learned mode of the batch: two frames (two judge phases) equal the
    single-view renderer's learned mode bit for bit; fine-tuning on the judged
    tiles returns a finite loss and sampled error and changes the network."""
    torch = cuda
    import ctypes as C
    from legitengine_gb300.train_reconstructor import DEFAULT_WEIGHTS
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    sizes = [(320, 240, 8, 0, 64), (256, 160, 16, 0, 64), (200, 136, 12, 0, 32)]
    specs = []
    for k, (W, H, R, SR, cap) in enumerate(sizes):
        view, t = _inputs(gi, torch, 500 + k, W, H, light)
        t["out_lit"] = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        t["out_indirect"] = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        specs.append(dict(view=view, march=gi.GiMarchParams(R, cap, 4, SR), **t))
    net = gi.Mlp(seed=None)
    net.load(str(DEFAULT_WEIGHTS))
    torch.cuda.synchronize()
    b = gi.Batch(specs, tile_rows=4)
    b.set_learned(net, few_dirs=2, few_step_dirs=16, judge_every=4, threshold=0.25)
    rs = []
    for (W, H, R, SR, cap) in sizes:
        r = gi.Renderer(W, H, dirs=R, step_cap=cap, bounces=1, bilateral=True, step_dirs=SR)
        r.set_learned(net, few_dirs=2, few_step_dirs=16, judge_every=4, threshold=0.25)
        rs.append(r)
    stream = torch.cuda.Stream()
    for frame in range(2):
        b.render(C.c_void_p(stream.cuda_stream))
        stream.synchronize()
        for s, r, (W, H, R, SR, cap) in zip(specs, rs, sizes):
            lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
            ind = torch.empty_like(lit)
            r.render(s["view"], s["albedo"], s["normal"], s["moments"], s["ndc"], s["direct"], lit, ind)
            torch.cuda.synchronize()
            assert torch.equal(ind, s["out_indirect"]), (frame, W, H)
            assert torch.equal(lit, s["out_lit"]), (frame, W, H)
    judged, fell = b.stats()
    assert judged == sum(r.stats()[0] for r in rs) and judged > 0
    assert fell == sum(r.stats()[1] for r in rs)
    before = net.get_params()
    loss, err = b.finetune(net, target_dirs=32, lr=1e-5)
    assert np.isfinite(loss) and loss >= 0 and 0 <= err < 1, (loss, err)
    assert not np.array_equal(before, net.get_params())
    for r in rs:
        r.close()
    b.close()


def test_online_finetuning_reduces_the_sampled_error(gi, cuda):
    """Online fine-tuning of a learned batch: an untrained network in a batch of two
    views takes one Adam step per frame on the judged tiles against their
    256-direction march.  Its sampled error falls and closes at least half of the gap
    to the shipped (offline-trained) network's error on the same batch, measured
    with fine-tuning steps of learning rate 0 (which leave the network unchanged)."""
    torch = cuda
    import ctypes as C
    from legitengine_gb300.train_reconstructor import DEFAULT_WEIGHTS
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    specs = []
    for k, (W, H) in enumerate(((256, 192), (192, 160))):
        view, t = _inputs(gi, torch, 700 + k, W, H, light)
        t["out_lit"] = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        specs.append(dict(view=view, march=gi.GiMarchParams(8, 64, 4, 0), **t))
    torch.cuda.synchronize()
    b = gi.Batch(specs, tile_rows=4)
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)

    def run(net, frames, lr):
        b.set_learned(net, few_dirs=1, few_step_dirs=32, judge_every=2, threshold=10.0)  # no fallback
        errs = []
        for _ in range(frames):
            b.render(sp)
            loss, err = b.finetune(net, target_dirs=256, lr=lr, stream=sp)
            assert np.isfinite(loss) and np.isfinite(err)
            errs.append(err)
        return errs

    shipped = gi.Mlp(seed=None)
    shipped.load(str(DEFAULT_WEIGHTS))
    before = shipped.get_params()
    floor = float(np.mean(run(shipped, 4, 0.0)))
    assert np.array_equal(before, shipped.get_params())
    errs = run(gi.Mlp(seed=123), 60, 3e-3)
    first, last = float(np.mean(errs[:4])), float(np.mean(errs[-4:]))
    print(f"online fine-tuning: sampled error {first:.4f} -> {last:.4f} (shipped network {floor:.4f})")
    assert last < first
    assert last - floor < 0.5 * (first - floor)
    b.close()
