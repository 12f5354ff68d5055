"""GPU parity: every CUDA pass, called through the C ABI, against the CPU oracle
on the same seeded inputs.

Bars: integer maps, mip geometry and the mip/blur/permutation payloads are
bit-exact; radiance is within 1e-3 relative per pixel (floor 1e-6) of the fp32
oracle.  The fp32 paths are written to the same evaluation order as the oracle,
so the tests also report (and bound) the fraction of bit-identical values.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

RADIANCE_RTOL = 1e-3


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def _random_image(rng, w, h, ch, depth_like=False):
    if depth_like:
        d = rng.uniform(0.2, 2.0, (h, w)).astype(np.float32)
        cols = [d, d + rng.uniform(0.0, 0.1, (h, w)).astype(np.float32), rng.uniform(0, 1, (h, w)),
                np.zeros((h, w))]
        return np.ascontiguousarray(np.stack(cols[:ch], -1).astype(np.float32))
    return rng.uniform(-1.0, 4.0, (h, w, ch)).astype(np.float32)


@pytest.mark.parametrize("w,h", [(512, 512), (1920, 1080), (37, 23), (3, 2), (640, 480)])
@pytest.mark.parametrize("ch", [1, 2, 4])
@pytest.mark.parametrize("filt", [0, 1])
def test_mips_bit_exact(gi, oracle, cuda, w, h, ch, filt):
    torch = cuda
    rng = np.random.default_rng(w * 7 + h + ch + filt)
    img = _random_image(rng, w, h, ch, depth_like=filt == 1)
    n = gi.mip_level_count(w, h, 10)
    lv = gi.alloc_pyramid(w, h, ch, n)
    lv[0].copy_(dev(torch, img))
    gi.build_mips(lv, ch, filt)
    ref = oracle.mip_chain(img, n, filt)
    for k in range(1, n):
        np.testing.assert_array_equal(host(lv[k]), ref[k], err_msg=f"level {k}")


@pytest.mark.parametrize("w,h", [(512, 512), (37, 23), (1920, 1080)])
@pytest.mark.parametrize("ch", [1, 2, 4])
@pytest.mark.parametrize("radius", [0, 1, 2, 3])
def test_blur_bit_exact(gi, oracle, cuda, w, h, ch, radius):
    torch = cuda
    img = _random_image(np.random.default_rng(3), w, h, ch)
    src = dev(torch, img)
    dst = torch.empty_like(src)
    gi.blur(src, dst, radius)
    np.testing.assert_array_equal(host(dst), oracle.blur(img, radius))


def test_blur_pyramid_bit_exact_and_aliased_level0(gi, oracle, cuda):
    torch = cuda
    w, h = 1920, 1080
    img = _random_image(np.random.default_rng(4), w, h, 4)
    n = gi.mip_level_count(w, h, 10)
    lv = gi.alloc_pyramid(w, h, 4, n)
    lv[0].copy_(dev(torch, img))
    gi.build_mips(lv, 4)
    out = [lv[0]] + gi.alloc_pyramid(w, h, 4, n)[1:]
    gi.blur_pyramid(lv, out)
    ref = oracle.blur_pyramid(oracle.mip_chain(img, n))
    for k in range(n):
        np.testing.assert_array_equal(host(out[k]), ref[k], err_msg=f"level {k}")


@pytest.mark.parametrize("w,h", [(1920, 1080), (512, 512), (16, 8)])
@pytest.mark.parametrize("ch", [1, 2, 4])
def test_deinterleave_interleave_bit_exact(gi, oracle, cuda, w, h, ch):
    torch = cuda
    img = _random_image(np.random.default_rng(5), w, h, ch)
    src = dev(torch, img)
    d = torch.empty_like(src)
    back = torch.empty_like(src)
    gi.deinterleave(src, d)
    np.testing.assert_array_equal(host(d), oracle.deinterleave(img))
    gi.interleave(d, back)
    np.testing.assert_array_equal(host(back), img)
    np.testing.assert_array_equal(host(back), oracle.interleave(oracle.deinterleave(img)))


def _gpu_pyramids(gi, torch, direct, moments, L):
    w, h = direct.shape[1], direct.shape[0]
    ll = gi.alloc_pyramid(w, h, 4, L)
    dl = gi.alloc_pyramid(w, h, 2, L)
    ll[0].copy_(dev(torch, direct))
    dl[0].copy_(dev(torch, moments))
    gi.build_mips(ll, 4)
    gi.build_mips(dl, 2)
    lb = [ll[0]] + gi.alloc_pyramid(w, h, 4, L)[1:]
    db = [dl[0]] + gi.alloc_pyramid(w, h, 2, L)[1:]
    gi.blur_pyramid(ll, lb)
    gi.blur_pyramid(dl, db)
    return lb, db


def _report(name, got, ref):
    e = rel_err(got, ref)
    exact = float(np.mean(got == ref))
    print(f"{name}: max rel {e.max():.3g}, bit-identical {exact * 100:.3f}%")
    return e, exact


@pytest.mark.parametrize("dirs,cap", [(4, 0), (8, 32), (16, 64), (2, 0)])
def test_march_small_frame(gi, oracle, cuda, scene_small, dirs, cap):
    torch = cuda
    s = scene_small
    gb, direct, view = s["gb"], s["direct"], s["view"]
    L = gi.mip_level_count(view.width, view.height, 10)
    lb, db = _gpu_pyramids(gi, torch, direct, gb["moments"], L)
    out = torch.empty((view.height, view.width, 4), dtype=torch.float32, device="cuda")
    gi.march(view, gi.GiMarchParams(dirs, cap, 4), lb, db, dev(torch, gb["normal"]), dev(torch, gb["ndc"]), out)
    ref_lb = oracle.blur_pyramid(oracle.mip_chain(direct, L))
    ref_db = oracle.blur_pyramid(oracle.mip_chain(gb["moments"], L))
    ref, _ = oracle.march(view, dirs, cap, ref_lb, ref_db, gb["normal"], gb["ndc"])
    e, exact = _report(f"march R={dirs}", host(out), ref)
    assert e.max() <= RADIANCE_RTOL
    assert exact >= 0.999


@pytest.mark.parametrize("dirs,cap", [(8, 32), (16, 64)])
def test_march_soft_occlusion(gi, oracle, cuda, scene_small, dirs, cap):
    """GI_OCCLUSION_SOFT (the depth-variance horizon) against its oracle restatement
    (SoftHorizon in gi_oracle.cpp): the same bar as the hard march; the FP32 oracle
    against its FP64 evaluation on the frame; and the soft result differs from the
    hard one (the variance is live)."""
    torch = cuda
    s = scene_small
    gb, direct, view = s["gb"], s["direct"], s["view"]
    L = gi.mip_level_count(view.width, view.height, 10)
    lb, db = _gpu_pyramids(gi, torch, direct, gb["moments"], L)
    out = torch.empty((view.height, view.width, 4), dtype=torch.float32, device="cuda")
    hard = torch.empty_like(out)
    nrm, ndc = dev(torch, gb["normal"]), dev(torch, gb["ndc"])
    gi.march(view, gi.GiMarchParams(dirs, cap, 4, 0, 0, gi.GI_OCCLUSION_SOFT), lb, db, nrm, ndc, out)
    gi.march(view, gi.GiMarchParams(dirs, cap, 4, 0, 0, gi.GI_OCCLUSION_HARD), lb, db, nrm, ndc, hard)
    ref_lb = oracle.blur_pyramid(oracle.mip_chain(direct, L))
    ref_db = oracle.blur_pyramid(oracle.mip_chain(gb["moments"], L))
    ref, _ = oracle.march(view, dirs, cap, ref_lb, ref_db, gb["normal"], gb["ndc"], soft=True)
    e, exact = _report(f"soft march R={dirs} cap={cap}", host(out), ref)
    assert e.max() <= RADIANCE_RTOL and exact >= 0.999
    r64, _ = oracle.march(view, dirs, cap, ref_lb, ref_db, gb["normal"], gb["ndc"], soft=True, dtype=np.float64)
    d64 = np.abs(ref[..., :3] - r64[..., :3]).sum() / np.abs(r64[..., :3]).sum()
    changed = np.abs(host(out)[..., :3] - host(hard)[..., :3]).sum() / np.abs(host(hard)[..., :3]).sum()
    print(f"soft R={dirs}: fp32 vs fp64 frame rel L1 {d64:.2e}; soft vs hard {changed:.3e}")
    assert d64 < 1e-3 and changed > 1e-4


@pytest.mark.parametrize("dirs,cap,step_dirs", [(8, 32, 0), (16, 64, 0), (2, 64, 32)])
def test_march_fast_precision(gi, oracle, cuda, scene_small, dirs, cap, step_dirs):
    """GI_MARCH_FAST (hardware rsqrt and reciprocal, a fitted atan, fused
    multiply-adds in the step loop) against the exact fp32 oracle: radiance within
    1e-3 relative per pixel and channel (floor 1e-6, as for the exact path)."""
    torch = cuda
    s = scene_small
    gb, direct, view = s["gb"], s["direct"], s["view"]
    L = gi.mip_level_count(view.width, view.height, 10)
    lb, db = _gpu_pyramids(gi, torch, direct, gb["moments"], L)
    out = torch.empty((view.height, view.width, 4), dtype=torch.float32, device="cuda")
    gi.march(view, gi.GiMarchParams(dirs, cap, 4, step_dirs, gi.GI_MARCH_FAST), lb, db, dev(torch, gb["normal"]),
             dev(torch, gb["ndc"]), out)
    ref_lb = oracle.blur_pyramid(oracle.mip_chain(direct, L))
    ref_db = oracle.blur_pyramid(oracle.mip_chain(gb["moments"], L))
    ref, _ = oracle.march(view, dirs, cap, ref_lb, ref_db, gb["normal"], gb["ndc"], step_dirs=step_dirs)
    e, exact = _report(f"fast march R={dirs} cap={cap} step_dirs={step_dirs}", host(out), ref)
    assert e.max() <= RADIANCE_RTOL
    assert np.all(host(out)[..., 3] == 1.0)


@pytest.mark.parametrize("dirs,step_dirs", [(2, 32), (4, 16)])
def test_march_step_dirs(gi, oracle, cuda, scene_small, dirs, step_dirs):
    """Few directions stepped at a denser angular spacing (the learned method's input)."""
    torch = cuda
    s = scene_small
    gb, direct, view = s["gb"], s["direct"], s["view"]
    L = gi.mip_level_count(view.width, view.height, 10)
    lb, db = _gpu_pyramids(gi, torch, direct, gb["moments"], L)
    out = torch.empty((view.height, view.width, 4), dtype=torch.float32, device="cuda")
    gi.march(view, gi.GiMarchParams(dirs, 64, 4, step_dirs), lb, db, dev(torch, gb["normal"]),
             dev(torch, gb["ndc"]), out)
    ref_lb = oracle.blur_pyramid(oracle.mip_chain(direct, L))
    ref_db = oracle.blur_pyramid(oracle.mip_chain(gb["moments"], L))
    ref, _ = oracle.march(view, dirs, 64, ref_lb, ref_db, gb["normal"], gb["ndc"], step_dirs=step_dirs)
    e, exact = _report(f"march R={dirs} step_dirs={step_dirs}", host(out), ref)
    assert e.max() <= RADIANCE_RTOL and exact >= 0.999


def test_march_deinterleaved_form(gi, oracle, cuda, scene_small):
    """A5 -> A7' -> A6 equals the oracle's interleaved-form march, and tracks A7."""
    torch = cuda
    s = scene_small
    gb, direct, view = s["gb"], s["direct"], s["view"]
    L = gi.mip_level_count(view.width, view.height, 10)
    lb, db = _gpu_pyramids(gi, torch, direct, gb["moments"], L)
    nrm, ndc = dev(torch, gb["normal"]), dev(torch, gb["ndc"])
    nrm_d, ndc_d = torch.empty_like(nrm), torch.empty_like(ndc)
    gi.deinterleave(nrm, nrm_d)
    gi.deinterleave(ndc, ndc_d)
    out_d = torch.empty((view.height, view.width, 4), dtype=torch.float32, device="cuda")
    params = gi.GiMarchParams(8, 32, 4)
    gi.march(view, params, lb, db, nrm_d, ndc_d, out_d, deinterleaved=True)
    out = torch.empty_like(out_d)
    gi.interleave(out_d, out)
    ref_lb = oracle.blur_pyramid(oracle.mip_chain(direct, L))
    ref_db = oracle.blur_pyramid(oracle.mip_chain(gb["moments"], L))
    ref_d = oracle.march_deinterleaved(view, 8, 32, ref_lb, ref_db, oracle.deinterleave(gb["normal"]),
                                       oracle.deinterleave(gb["ndc"]))
    e, exact = _report("march A7'", host(out_d), ref_d)
    assert e.max() <= RADIANCE_RTOL and exact >= 0.999
    full, _ = oracle.march(view, 8, 32, ref_lb, ref_db, gb["normal"], gb["ndc"])
    np.testing.assert_array_equal(host(out), oracle.interleave(host(out_d)))
    assert rel_err(host(out)[..., :3], full[..., :3], floor=1e-2).max() < 1e-2


def test_inputs_and_march_1080p_sampled(gi, oracle, cuda):
    """1920x1080, 64 boxes + 16 spheres, R = 16, cap 64: G-buffer, shadow, direct light on the GPU
    against the oracle, then the march on 4096 sampled pixels (full-frame oracle is minutes of CPU)."""
    torch = cuda
    prims = gi.scene_generate(2000, 64, 16)
    view = gi.view_from_camera(gi.camera_spline(2, 5, 64), 1920, 1080)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    pd, npr = gi.prims_to_device(prims)
    W, H = 1920, 1080
    t = {k: torch.empty((H, W, c), dtype=torch.float32, device="cuda")
         for k, c in (("albedo", 4), ("emissive", 4), ("normal", 4), ("moments", 2), ("ndc", 1))}
    gi.gbuffer(view, pd, npr, t["albedo"], t["emissive"], t["normal"], t["moments"], t["ndc"])
    sm = torch.empty((1024, 1024, 1), dtype=torch.float32, device="cuda")
    gi.shadow_map(light, pd, npr, sm)
    direct = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    gi.direct_light(view, light, t["albedo"], t["emissive"], t["normal"], t["ndc"], sm, direct)
    gb = oracle.gbuffer(view, prims)
    for k in t:
        g = host(t[k])
        assert np.mean(g == gb[k]) > 0.9999, k
        assert rel_err(g, gb[k]).max() < 1e-5, k
    osm = oracle.shadow_map(light, prims)
    assert np.mean(host(sm) == osm) > 0.9999
    od = oracle.direct_light(view, light, gb, osm)
    e, exact = _report("direct", host(direct), od)
    assert exact > 0.999
    # March on sampled pixels, same inputs on both sides.
    L = gi.mip_level_count(W, H, 10)
    lb, db = _gpu_pyramids(gi, torch, host(direct), gb["moments"], L)
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    gi.march(view, gi.GiMarchParams(16, 64, 4), lb, db, dev(torch, gb["normal"]), dev(torch, gb["ndc"]), out)
    rng = np.random.default_rng(9)
    pix = np.stack([rng.integers(0, W, 4096), rng.integers(0, H, 4096)], -1)
    pix = np.concatenate([pix, [[0, 0], [W - 1, H - 1], [W // 2, H // 2], [W - 1, 0]]])
    ref_lb = oracle.blur_pyramid(oracle.mip_chain(host(direct), L))
    ref_db = oracle.blur_pyramid(oracle.mip_chain(gb["moments"], L))
    ref, _ = oracle.march(view, 16, 64, ref_lb, ref_db, gb["normal"], gb["ndc"], pixels=pix)
    got = host(out)[pix[:, 1], pix[:, 0]]
    e, exact = _report("march 1080p", got, ref)
    assert e.max() <= RADIANCE_RTOL and exact >= 0.999


def test_filters_bit_exact(gi, oracle, cuda, scene_small):
    torch = cuda
    gb = scene_small["gb"]
    rng = np.random.default_rng(11)
    h, w = gb["normal"].shape[:2]
    ind = rng.uniform(0, 2, (h, w, 4)).astype(np.float32)
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    gi.bilateral(dev(torch, ind), dev(torch, gb["moments"]), dev(torch, gb["normal"]), out)
    e, exact = _report("bilateral", host(out), oracle.bilateral(ind, gb["moments"], gb["normal"]))
    assert e.max() <= RADIANCE_RTOL and exact >= 0.999
    # an odd size: partial tiles in x and y, a thread's second row past the bottom edge
    ci, cm, cn = (np.ascontiguousarray(a[:45, :67]) for a in (ind, gb["moments"], gb["normal"]))
    co = torch.empty((45, 67, 4), dtype=torch.float32, device="cuda")
    gi.bilateral(dev(torch, ci), dev(torch, cm), dev(torch, cn), co)
    e, exact = _report("bilateral 67x45", host(co), oracle.bilateral(ci, cm, cn))
    assert e.max() <= RADIANCE_RTOL and exact >= 0.999
    for r in (0, 2):
        gi.denoise(dev(torch, ind), dev(torch, gb["moments"]), dev(torch, gb["normal"]), out, r)
        e, exact = _report(f"denoise r={r}", host(out), oracle.denoise(ind, gb["moments"], r))
        assert exact >= 0.999 and e.max() <= RADIANCE_RTOL
    gi.final_gather(dev(torch, scene_small["direct"]), dev(torch, ind), dev(torch, gb["albedo"]), out)
    np.testing.assert_array_equal(host(out), oracle.final_gather(scene_small["direct"], ind, gb["albedo"]))


@pytest.mark.parametrize("bounces", [1, 2])
def test_renderer_end_to_end(gi, oracle, cuda, bounces):
    """The whole GI segment (mips, blur, march, bilateral, gather; 1 or 2 bounces) at 256x144,
    through the graph-captured renderer, against the oracle pipeline on the same G-buffer."""
    torch = cuda
    prims = gi.scene_generate(2000, 64, 16)
    view = gi.view_from_camera(gi.camera_spline(2, 9, 64), 256, 144)
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    gb = oracle.gbuffer(view, prims)
    direct = oracle.direct_light(view, light, gb, oracle.shadow_map(light, prims))
    r = gi.Renderer(256, 144, dirs=16, step_cap=64, bounces=bounces)
    lit = torch.empty((144, 256, 4), dtype=torch.float32, device="cuda")
    ind = torch.empty_like(lit)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        r.render(view, dev(torch, gb["albedo"]), dev(torch, gb["normal"]), dev(torch, gb["moments"]),
                 dev(torch, gb["ndc"]), dev(torch, direct), lit, ind)
    stream.synchronize()
    ref = oracle.render_frame(view, gb, direct, 16, 64, bounces=bounces)
    e, exact = _report(f"renderer lit b={bounces}", host(lit), ref["lit"])
    assert e.max() <= RADIANCE_RTOL and exact >= 0.999
    e, _ = _report(f"renderer indirect b={bounces}", host(ind), ref[f"indirect{bounces - 1}"])
    assert e.max() <= RADIANCE_RTOL


@pytest.mark.parametrize("fast", [False, True])
def test_renderer_three_bounces_odd_size(gi, oracle, cuda, fast):
    """Three bounces at 130x77 (sub-images of uneven size: the march record's
    interleaved indexing with partial rows and columns): bounces 2 and 3 re-light
    bounce 1's recorded march.  Exact precision: bit-identical to the oracle's
    three marches; fast: within 1e-3 of the exact renderer."""
    torch = cuda
    W, H = 130, 77
    prims = gi.scene_generate(2300, 32, 8)
    view = gi.view_from_camera(gi.camera_spline(23, 3, 64), W, H)
    light = gi.view_from_camera(gi.scene_light(), 256, 256)
    gb = oracle.gbuffer(view, prims)
    direct = oracle.direct_light(view, light, gb, oracle.shadow_map(light, prims))
    args = [dev(torch, x) for x in (gb["albedo"], gb["normal"], gb["moments"], gb["ndc"], direct)]
    outs = {}
    for prec in ([gi.GI_MARCH_EXACT, gi.GI_MARCH_FAST] if fast else [gi.GI_MARCH_EXACT]):
        r = gi.Renderer(W, H, dirs=12, step_cap=48, bounces=3, precision=prec)
        lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        r.render(view, *args, lit)
        torch.cuda.synchronize()
        outs[prec] = host(lit)
        r.close()
    if fast:
        e = rel_err(outs[gi.GI_MARCH_FAST], outs[gi.GI_MARCH_EXACT], floor=1e-3 * np.abs(outs[0]).mean())
        print(f"3 bounces fast vs exact: max rel {e.max():.3g}")
        assert e.max() <= RADIANCE_RTOL
    else:
        ref = oracle.render_frame(view, gb, direct, 12, 48, bounces=3)
        e, exact = _report("renderer lit b=3 130x77", outs[gi.GI_MARCH_EXACT], ref["lit"])
        assert e.max() <= RADIANCE_RTOL and exact >= 0.999


def test_renderer_graph_replay_and_host_path(gi, cuda):
    """Consecutive frames with different views update the captured graph; the host-buffer entry
    point gives the same image as the device one; the library counts its launches."""
    torch = cuda
    prims = gi.scene_generate(3000, 16, 4)
    pd, npr = gi.prims_to_device(prims)
    W, H = 320, 240
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    r = gi.Renderer(W, H, dirs=8, step_cap=32, bounces=2)
    stream = torch.cuda.Stream()
    outs = []
    for f in (0, 17, 0):
        view = gi.view_from_camera(gi.camera_spline(3, f, 64), W, H)
        t = {k: torch.empty((H, W, c), dtype=torch.float32, device="cuda")
             for k, c in (("albedo", 4), ("emissive", 4), ("normal", 4), ("moments", 2), ("ndc", 1))}
        sm = torch.empty((512, 512, 1), dtype=torch.float32, device="cuda")
        direct = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        with torch.cuda.stream(stream):
            gi.gbuffer(view, pd, npr, t["albedo"], t["emissive"], t["normal"], t["moments"], t["ndc"])
            gi.shadow_map(light, pd, npr, sm)
            gi.direct_light(view, light, t["albedo"], t["emissive"], t["normal"], t["ndc"], sm, direct)
            lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
            n0 = gi.lib().gi_launch_count()
            r.render(view, t["albedo"], t["normal"], t["moments"], t["ndc"], direct, lit)
            assert gi.lib().gi_launch_count() - n0 >= 10
        stream.synchronize()
        outs.append(host(lit))
        hl = torch.empty((H, W, 4), dtype=torch.float32).pin_memory()
        args = [x.cpu().pin_memory() for x in (t["albedo"], t["normal"], t["moments"], t["ndc"], direct)]
        r.render_host(view, *args, hl, stream=__import__("ctypes").c_void_p(stream.cuda_stream))
        np.testing.assert_array_equal(hl.numpy(), outs[-1])
    np.testing.assert_array_equal(outs[0], outs[2])
    assert not np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("dirs,step_dirs", [(16, 0), (2, 32)])
def test_march_fast_precision_1080p(gi, oracle, cuda, dirs, step_dirs):
    """GI_MARCH_FAST on a full 1080p frame of the bench scene.

    Against the exact path: the frame's relative L1 difference is bounded, and at
    the plain workload's 16 directions every pixel is within 1e-3 relative (floor
    1e-3 of the frame's mean radiance).  Against the FP64 re-evaluation of the same
    estimator, on 2048 random pixels and on the 512 where fast and exact differ
    most: the fast path is as accurate as the exact fp32 path (mean relative error
    within 2 % of the exact path's, its 99th percentile within 5 % -- a percentile
    of the 512 most-different pixels is a noisy statistic -- plus 1e-5 each; the
    largest error no more than 1e-3 above the exact path's largest).

    The exact path itself is not within 1e-3 of FP64 everywhere (its mean relative
    error on random pixels is ~6e-4 at 2 directions): its integer decisions (step
    counts, horizon updates, texel and level selection) can fall the other way in
    double, and where the radiance is a cancelling sum of light and ambient terms,
    or a sample lies close to the centre point, two valid fp32 evaluation orders
    differ by more than 1e-3 of the result.  Few-direction frames have such
    pixels, so there the two fp32 paths are compared through FP64, not pixel by pixel."""
    torch = cuda
    from legitengine_gb300.train_reconstructor import Frame
    W, H = 1920, 1080
    fr = Frame(gi, torch, W, H)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    prims = gi.scene_generate(20002, 64, 16)
    pd, npr = gi.prims_to_device(prims)
    fr.inputs(pd, npr, gi.view_from_camera(gi.camera_spline(20000, 32, 64, prims), W, H), light)
    a = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    gi.march(fr.view, gi.GiMarchParams(dirs, 64, 4, step_dirs, gi.GI_MARCH_EXACT), fr.lb, fr.db, fr.normal,
             fr.ndc, a)
    gi.march(fr.view, gi.GiMarchParams(dirs, 64, 4, step_dirs, gi.GI_MARCH_FAST), fr.lb, fr.db, fr.normal,
             fr.ndc, b)
    x, y = host(b)[..., :3].astype(np.float64), host(a)[..., :3].astype(np.float64)
    frame_l1 = np.abs(x - y).sum() / np.abs(y).sum()
    floor = 1e-3 * np.abs(y).mean()
    vs_exact = rel_err(x, y, floor=floor).max(-1)
    rng = np.random.default_rng(dirs)
    rand = rng.choice(W * H, 2048, replace=False)
    worst = np.argsort(vs_exact.ravel())[-512:]
    pick = np.unique(np.concatenate([worst, rand]))
    pix = np.stack([pick % W, pick // W], 1).astype(np.int32)
    lb = [host(t) for t in fr.lb]
    db = [host(t) for t in fr.db]
    ref, _ = oracle.march(fr.view, dirs, 64, lb, db, host(fr.normal), host(fr.ndc), pixels=pix, dtype=np.float64,
                          step_dirs=step_dirs)
    ref = dict(zip(pick.tolist(), np.asarray(ref, np.float64).reshape(-1, 4)[:, :3]))

    def errors(idx):
        r = np.stack([ref[i] for i in idx.tolist()])
        den = np.maximum(np.abs(r), floor)
        return (np.abs(x.reshape(-1, 3)[idx] - r) / den).ravel(), (np.abs(y.reshape(-1, 3)[idx] - r) / den).ravel()

    print(f"fast 1080p R={dirs} s={step_dirs}: frame rel L1 vs exact {frame_l1:.2e}; max vs exact "
          f"{vs_exact.max():.2e}, pixels above 1e-3 {(vs_exact > RADIANCE_RTOL).sum()}")
    for name, idx in (("random", rand), ("worst", worst)):
        ef, ee = errors(idx)
        print(f"  vs fp64, {len(idx)} {name} px: fast mean {ef.mean():.3e} p99 {np.quantile(ef, 0.99):.3e} max "
              f"{ef.max():.3e}; exact mean {ee.mean():.3e} p99 {np.quantile(ee, 0.99):.3e} max {ee.max():.3e}")
        assert ef.mean() <= 1.02 * ee.mean() + 1e-5
        assert np.quantile(ef, 0.99) <= 1.05 * np.quantile(ee, 0.99) + 1e-5
        assert ef.max() <= ee.max() + RADIANCE_RTOL
    assert frame_l1 < 1e-5
    if dirs >= 16:
        assert vs_exact.max() <= RADIANCE_RTOL


def test_small_room_512_end_to_end(gi, oracle, cuda):
    """The small plain workload at its own sizes: a 512x512 frame of the seeded
    16-box room (scene seed 1000), 1024^2 shadow map, 8 directions, 32 steps, one
    bounce, the 5x5 bilateral.  The input stages on the GPU, then the graph-captured renderer, each
    against the oracle on the same inputs."""
    torch = cuda
    W = H = 512
    prims = gi.scene_generate(1000, 16, 0)
    view = gi.view_from_camera(gi.camera_spline(1000, 0, 64, prims), W, H)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    pd, npr = gi.prims_to_device(prims)
    t = {k: torch.empty((H, W, c), dtype=torch.float32, device="cuda")
         for k, c in (("albedo", 4), ("emissive", 4), ("normal", 4), ("moments", 2), ("ndc", 1), ("direct", 4))}
    sm = torch.empty((1024, 1024, 1), dtype=torch.float32, device="cuda")
    gi.gbuffer(view, pd, npr, t["albedo"], t["emissive"], t["normal"], t["moments"], t["ndc"])
    gi.shadow_map(light, pd, npr, sm)
    gi.direct_light(view, light, t["albedo"], t["emissive"], t["normal"], t["ndc"], sm, t["direct"])
    gb = oracle.gbuffer(view, prims)
    osm = oracle.shadow_map(light, prims)
    od = oracle.direct_light(view, light, gb, osm)
    for k in ("albedo", "normal", "moments", "ndc"):
        assert np.mean(host(t[k]) == gb[k]) > 0.9999, k
    assert np.mean(host(sm) == osm) > 0.9999
    e, exact = _report("512x512 direct", host(t["direct"]), od)
    assert exact > 0.999
    r = gi.Renderer(W, H, dirs=8, step_cap=32, bounces=1)
    lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    ind = torch.empty_like(lit)
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        r.render(view, dev(torch, gb["albedo"]), dev(torch, gb["normal"]), dev(torch, gb["moments"]),
                 dev(torch, gb["ndc"]), dev(torch, od), lit, ind)
    stream.synchronize()
    ref = oracle.render_frame(view, gb, od, 8, 32, bounces=1)
    e, exact = _report("512x512 lit", host(lit), ref["lit"])
    assert e.max() <= RADIANCE_RTOL and exact >= 0.999
    e, exact = _report("512x512 indirect", host(ind), ref["indirect0"])
    assert e.max() <= RADIANCE_RTOL and exact >= 0.999
    r.close()


def test_renderer_fast_precision_tracks_exact(gi, oracle, cuda):
    """The renderer in GI_MARCH_FAST (fast march and bilateral, two bounces) against
    the exact renderer on the same frame: frame relative L1 below 1e-5 and every
    value within 1e-3 relative (floor 1e-3 of the frame's mean radiance)."""
    torch = cuda
    prims = gi.scene_generate(2000, 64, 16)
    view = gi.view_from_camera(gi.camera_spline(2, 9, 64), 256, 144)
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    gb = oracle.gbuffer(view, prims)
    direct = oracle.direct_light(view, light, gb, oracle.shadow_map(light, prims))
    ins = [dev(torch, gb["albedo"]), dev(torch, gb["normal"]), dev(torch, gb["moments"]), dev(torch, gb["ndc"]),
           dev(torch, direct)]
    out = {}
    for prec in (gi.GI_MARCH_EXACT, gi.GI_MARCH_FAST):
        r = gi.Renderer(256, 144, dirs=16, step_cap=64, bounces=2, precision=prec)
        lit = torch.empty((144, 256, 4), dtype=torch.float32, device="cuda")
        r.render(view, *ins, lit)
        torch.cuda.synchronize()
        out[prec] = host(lit)[..., :3].astype(np.float64)
        r.close()
    x, y = out[gi.GI_MARCH_FAST], out[gi.GI_MARCH_EXACT]
    l1 = np.abs(x - y).sum() / np.abs(y).sum()
    e = rel_err(x, y, floor=1e-3 * np.abs(y).mean())
    print(f"renderer fast vs exact: frame rel L1 {l1:.2e}, max rel {e.max():.2e}")
    assert l1 < 1e-5 and e.max() <= RADIANCE_RTOL


def _renderer_frames(gi, torch, oracle, W, H, seed, frame, n_prims=64, n_spheres=16):
    prims = gi.scene_generate(seed, n_prims, n_spheres)
    view = gi.view_from_camera(gi.camera_spline(seed % 97, frame, 64), W, H)
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    gb = oracle.gbuffer(view, prims)
    direct = oracle.direct_light(view, light, gb, oracle.shadow_map(light, prims))
    return view, [dev(torch, x) for x in (gb["albedo"], gb["normal"], gb["moments"], gb["ndc"], direct)]


def _render(gi, torch, view, ins, **kw):
    r = gi.Renderer(view.width, view.height, **kw)
    lit = torch.empty((view.height, view.width, 4), dtype=torch.float32, device="cuda")
    r.render(view, *ins, lit)
    torch.cuda.synchronize()
    r.close()
    return host(lit)[..., :3].astype(np.float64)


@pytest.mark.parametrize("bounces,W,H", [(2, 256, 144), (3, 130, 77)])
def test_renderer_texture_precision(gi, oracle, cuda, bounces, W, H):
    """GI_MARCH_TEXTURE (the fast loop with trilinear depth and light fetches by the
    texture units, 8-bit sub-texel and level weights; two and three bounces, so the
    recorded march and its replay both fetch through the textures): its distance to
    the exact renderer stays three orders of magnitude below the estimator's own
    error -- frame relative L1 below 1e-3, under 2 % of the values off by more than
    1e-2 -- and its error against a converged render (exact, 256 directions, no step
    cap) is the exact renderer's within 1 %."""
    torch = cuda
    view, ins = _renderer_frames(gi, torch, oracle, W, H, 2100 + bounces, 9)
    kw = dict(dirs=16, step_cap=64, bounces=bounces)
    y = _render(gi, torch, view, ins, precision=gi.GI_MARCH_EXACT, **kw)
    x = _render(gi, torch, view, ins, precision=gi.GI_MARCH_TEXTURE, **kw)
    conv = _render(gi, torch, view, ins, precision=gi.GI_MARCH_EXACT, dirs=256, step_cap=0, bounces=bounces)
    l1 = np.abs(x - y).sum() / np.abs(y).sum()
    rel = rel_err(x, y, floor=1e-3 * np.abs(y).mean())
    over = float(np.mean(rel > 1e-2))
    err_x = np.abs(x - conv).sum() / np.abs(conv).sum()
    err_y = np.abs(y - conv).sum() / np.abs(conv).sum()
    print(f"texture vs exact ({bounces} bounces): frame rel L1 {l1:.2e}, max rel {rel.max():.2e}, "
          f"over 1e-2 {over * 100:.3f}%; error vs converged {err_x:.5f} (exact {err_y:.5f})")
    assert l1 < 1e-3 and over < 0.02
    assert abs(err_x - err_y) <= 0.01 * err_y
    assert np.isfinite(x).all()


def test_march_texture_precision_through_the_abi(gi, oracle, cuda, scene_small):
    """gi_march with GI_MARCH_TEXTURE (caller-owned pyramids copied into the
    library's textures): within 1e-3 frame relative L1 of the software fast loop
    and not bit-identical to it (the taps come from the texture units); the same
    call repeated after a march of another size (the textures re-made) gives the
    same image bit for bit; the deinterleaved form refuses it."""
    torch = cuda
    s = scene_small
    view = s["view"]
    L = gi.mip_level_count(view.width, view.height, 10)
    lb, db = _gpu_pyramids(gi, torch, s["direct"], s["gb"]["moments"], L)
    nrm, ndc = dev(torch, s["gb"]["normal"]), dev(torch, s["gb"]["ndc"])

    def run(prec, v=view, l=lb, d=db, n=nrm, z=ndc):
        out = torch.empty((v.height, v.width, 4), dtype=torch.float32, device="cuda")
        gi.march(v, gi.GiMarchParams(8, 32, 4, 0, prec), l, d, n, z, out)
        torch.cuda.synchronize()
        return host(out)[..., :3].astype(np.float64)

    tex, fast = run(gi.GI_MARCH_TEXTURE), run(gi.GI_MARCH_FAST)
    l1 = np.abs(tex - fast).sum() / np.abs(fast).sum()
    print(f"gi_march texture vs fast: frame rel L1 {l1:.2e}")
    assert 0 < l1 < 1e-3
    other = _renderer_frames(gi, torch, oracle, 200, 120, 2301, 4)
    v2 = other[0]
    L2 = gi.mip_level_count(v2.width, v2.height, 10)
    lb2, db2 = _gpu_pyramids(gi, torch, host(other[1][4]), host(other[1][2]), L2)
    run(gi.GI_MARCH_TEXTURE, v2, lb2, db2, other[1][1], other[1][3])
    np.testing.assert_array_equal(run(gi.GI_MARCH_TEXTURE), tex)
    out = torch.empty((view.height, view.width, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(gi.GiError, match="GI_MARCH_TEXTURE"):
        gi.march(view, gi.GiMarchParams(8, 32, 4, 0, gi.GI_MARCH_TEXTURE), lb, db, nrm, ndc, out, deinterleaved=True)


def test_learned_renderer_texture_precision(gi, oracle, cuda):
    """The learned renderer with GI_MARCH_TEXTURE (few-ray march, judge march and
    fallbacks through the textures) stays within 5e-3 frame relative L1 of the
    learned renderer with the software fast loop."""
    torch = cuda
    from legitengine_gb300 import train_reconstructor as tr
    view, ins = _renderer_frames(gi, torch, oracle, 320, 192, 2207, 5)
    net = gi.Mlp(seed=None)
    net.load(str(tr.DEFAULT_WEIGHTS))
    out = {}
    for prec in (gi.GI_MARCH_FAST, gi.GI_MARCH_TEXTURE):
        r = gi.Renderer(320, 192, dirs=16, step_cap=64, bounces=2, precision=prec)
        r.set_learned(net, few_dirs=tr.DEFAULT_FEW_DIRS, few_step_dirs=tr.DEFAULT_FEW_STEP_DIRS)
        lit = torch.empty((192, 320, 4), dtype=torch.float32, device="cuda")
        r.render(view, *ins, lit)
        torch.cuda.synchronize()
        out[prec] = host(lit)[..., :3].astype(np.float64)
        r.close()
    x, y = out[gi.GI_MARCH_TEXTURE], out[gi.GI_MARCH_FAST]
    l1 = np.abs(x - y).sum() / np.abs(y).sum()
    print(f"learned texture vs learned fast: frame rel L1 {l1:.2e}")
    assert l1 < 5e-3 and np.isfinite(x).all()


def test_renderer_temporal_feedback(gi, oracle, cuda):
    """Temporal feedback (one march per frame over the previous frame's gathered
    image): the first frame equals the oracle's one-bounce frame on the direct
    light, the second the oracle's frame whose light is the first frame's image."""
    torch = cuda
    prims = gi.scene_generate(2000, 64, 16)
    light = gi.view_from_camera(gi.scene_light(), 512, 512)
    r = gi.Renderer(256, 144, dirs=16, step_cap=64, bounces=1, feedback=True)
    prev = None
    for k, frame in enumerate((9, 10)):
        view = gi.view_from_camera(gi.camera_spline(2, frame, 64), 256, 144)
        gb = oracle.gbuffer(view, prims)
        direct = oracle.direct_light(view, light, gb, oracle.shadow_map(light, prims))
        lit = torch.empty((144, 256, 4), dtype=torch.float32, device="cuda")
        r.render(view, dev(torch, gb["albedo"]), dev(torch, gb["normal"]), dev(torch, gb["moments"]),
                 dev(torch, gb["ndc"]), dev(torch, direct), lit)
        torch.cuda.synchronize()
        ref = oracle.render_frame(view, gb, direct, 16, 64, bounces=1, source=prev)
        e, exact = _report(f"feedback frame {k}", host(lit), ref["lit"])
        assert e.max() <= RADIANCE_RTOL and exact >= 0.999
        prev = host(lit)
    r.close()
    with pytest.raises(gi.GiError):
        gi.Renderer(64, 64, bounces=2, feedback=True)


@pytest.mark.parametrize("learned", [False, True])
def test_renderer_pipelined_host_frames(gi, cuda, learned):
    """gi_renderer_render_host_async over five frames of a camera path (inputs copied
    in while the previous frame renders, images copied out while the next renders)
    gives each frame's image bit for bit as the synchronous host path does; a frame's
    image is complete once the call two frames later has returned."""
    torch = cuda
    from legitengine_gb300 import train_reconstructor as tr
    W, H = 320, 184
    fr = tr.Frame(gi, torch, W, H)
    prims = gi.scene_generate(2100, 48, 8)
    pd, npr = gi.prims_to_device(prims)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    frames = []
    for k in range(5):
        view = gi.view_from_camera(gi.camera_spline(2100, 4 * k, 64, prims), W, H)
        fr.inputs(pd, npr, view, light)
        frames.append((view, [t.cpu().pin_memory() for t in (fr.albedo, fr.normal, fr.moments, fr.ndc, fr.direct)]))

    def renderer():
        r = gi.Renderer(W, H, dirs=16, step_cap=64, bounces=2, bilateral=True, precision=gi.GI_MARCH_FAST)
        if learned:
            net = gi.Mlp(seed=None)
            net.load(tr.DEFAULT_WEIGHTS)
            r.set_learned(net, few_dirs=tr.DEFAULT_FEW_DIRS, few_step_dirs=tr.DEFAULT_FEW_STEP_DIRS)
        return r

    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    r = renderer()
    want = []
    for view, ins in frames:
        out = torch.empty((H, W, 4), dtype=torch.float32).pin_memory()
        r.render_host(view, *ins, out, stream=sp)
        want.append(out.numpy().copy())
    r.close()
    r = renderer()
    outs = [torch.full((H, W, 4), -1.0, dtype=torch.float32).pin_memory() for _ in frames]
    for k, (view, ins) in enumerate(frames):
        r.render_host_async(view, *ins, outs[k], stream=sp)
        if k >= 2:
            np.testing.assert_array_equal(outs[k - 2].numpy(), want[k - 2])
    r.host_wait()
    for k in range(len(frames)):
        np.testing.assert_array_equal(outs[k].numpy(), want[k])
    assert not np.array_equal(want[0], want[1])
    r.close()


@pytest.mark.parametrize("learned", [False, True])
def test_renderer_pass_profiling(gi, cuda, learned):
    """Per-pass GPU times, as the reference's GPU profiler shows them: the frame's
    passes by their SetProfilerInfo names in recording order, contiguous
    non-decreasing intervals on the frame's stream; the image is unchanged."""
    torch = cuda
    from legitengine_gb300 import train_reconstructor as tr
    W, H = 320, 184
    fr = tr.Frame(gi, torch, W, H)
    prims = gi.scene_generate(2200, 48, 8)
    pd, npr = gi.prims_to_device(prims)
    view = gi.view_from_camera(gi.camera_spline(2200, 5, 64, prims), W, H)
    fr.inputs(pd, npr, view, gi.view_from_camera(gi.scene_light(), 1024, 1024))
    outs = []
    for profile in (False, True):
        r = gi.Renderer(W, H, dirs=16, step_cap=64, bounces=2, bilateral=True, precision=gi.GI_MARCH_FAST)
        if learned:
            net = gi.Mlp(seed=None)
            net.load(tr.DEFAULT_WEIGHTS)
            r.set_learned(net, few_dirs=tr.DEFAULT_FEW_DIRS, few_step_dirs=tr.DEFAULT_FEW_STEP_DIRS)
        r.set_profiling(profile)
        lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        r.render(view, fr.albedo, fr.normal, fr.moments, fr.ndc, fr.direct, lit)
        torch.cuda.synchronize()
        outs.append(host(lit))
        if profile:
            times = r.pass_times()
            names = [n for n, _, _ in times]
            print(" ".join(f"{n}:{b - a:.3f}" for n, a, b in times))
            want = "ReconstructPass" if learned else "IndirectLightPass"
            assert names.count(want) == 2 and names.count("GatheringPass") == 2
            if learned:
                assert names.count("FewRayPass") == 2 and names.count("JudgePass") == 2
            assert times[0][1] == 0.0
            for (_, a, b), (_, c, _) in zip(times, times[1:] + [(None, times[-1][2], None)]):
                assert 0.0 <= a <= b and abs(b - c) < 1e-6
            assert 0.0 < times[-1][2] < 1000.0
        r.close()
    np.testing.assert_array_equal(outs[0], outs[1])
