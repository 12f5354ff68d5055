"""The oracle pinned to the reference's own source: its GLSL passes compiled as
C++ against its own vendored glm (oracle/_ref, built by oracle/build_ref.py from
the reference checkout where it lies).

The oracle restates each shader under a fixed fp32 evaluation contract (the
library's; see oracle/glsl.h): its own transcendental functions, division as a
times the correctly rounded reciprocal, and the shader's per-pixel matrix
inverses hoisted to the host in double.  For the pin the oracle switches to the
C library's float functions and true division (oracle.set_libm) and takes the
matrices the shader itself derives from its uniforms (ref.shader_inverses): the
two then evaluate the same operations, and every test below asks for equal bits
-- colours, step counts and the mip level of every depth tap.  The contract's
own distance to the reference's evaluation (and both to the FP64 estimator) is
measured beside it.

These tests run where the reference checkout is (this repository's build
machine); elsewhere they skip.
"""
import copy

import numpy as np
import pytest

from conftest import rel_err

ref = pytest.importorskip("oracle.ref")
if not ref.available():
    pytest.skip("the reference checkout is not present", allow_module_level=True)


@pytest.fixture(scope="module")
def r(oracle):
    ref.lib()
    return ref


def _shader_view(ref, view):
    """The view with the inverses the indirect pass's shader computes itself."""
    ivp, iv = ref.shader_inverses(view.view, view.proj)
    v = copy.copy(view)
    for k in range(16):
        v.inv_view_proj[k] = float(ivp[k])
        v.inv_view[k] = float(iv[k])
    return v


class libm:
    def __init__(self, oracle):
        self.o = oracle

    def __enter__(self):
        self.o.set_libm(True)

    def __exit__(self, *exc):
        self.o.set_libm(False)


def _scene(gi, oracle, W, H, seed, spline, frame, boxes, spheres):
    prims = gi.scene_generate(seed, boxes, spheres)
    view = gi.view_from_camera(gi.camera_spline(spline, frame, 64), W, H)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    gb = oracle.gbuffer(view, prims)
    sm = oracle.shadow_map(light, prims)
    direct = oracle.direct_light(view, light, gb, sm)
    L = oracle.mip_level_count(W, H, 10)
    lb = oracle.blur_pyramid(oracle.mip_chain(direct, L))
    db = oracle.blur_pyramid(oracle.mip_chain(gb["moments"], L))
    return dict(view=view, light=light, gb=gb, sm=sm, direct=direct, lb=lb, db=db)


@pytest.fixture(scope="module")
def room512(gi, oracle):
    """BASELINE configuration 1's room: 512x512, 16 boxes."""
    return _scene(gi, oracle, 512, 512, 1000, 1, 3, 16, 0)


@pytest.fixture(scope="module")
def room1080(gi, oracle):
    """The headline configuration's room: 1920x1080, 64 boxes and 16 spheres."""
    return _scene(gi, oracle, 1920, 1080, 2000, 2, 5, 64, 16)


@pytest.mark.parametrize("w,h", [(512, 512), (37, 23), (1920, 1080)])
def test_mip_blur_permute_equal_the_reference_shaders(r, oracle, w, h):
    """Common/mipLevelBuilder.frag (average and "Depth" modes),
    Common/blurLayerBuilder.frag (radius 0 and 2), Common/deinterleave.frag and
    Common/interleave.frag: bit-identical, odd sizes included."""
    rng = np.random.default_rng(w * 7 + h)
    img = rng.uniform(0.05, 3.0, (h, w, 4)).astype(np.float32)
    assert np.array_equal(r.mip_level(img, 0), oracle.mip_level(img, 0))
    with libm(oracle):  # the Depth mode divides: true division, as the shader
        assert np.array_equal(r.mip_level(img, 1), oracle.mip_level(img, 1))
    for radius in (0, 2):
        assert np.array_equal(r.blur(img, radius), oracle.blur(img, radius))
    if w % 4 == 0 and h % 4 == 0:
        assert np.array_equal(r.permute(img, False), oracle.deinterleave(img))
        assert np.array_equal(r.permute(img, True), oracle.interleave(img))


def test_camera_and_projection_equal_glm(gi, r):
    """gi_view_from_camera against the matrices the reference builds with glm
    (Scene.h:30-33, SSVGIRenderer.h:54-59: view = inverse(translate * rotate *
    rotate), proj = perspective * scale(1, -1, -1), radians, depth [0, 1]): the
    library evaluates them in double and rounds once, glm in float; they agree to
    a few ulp of the matrices' largest entries (glm's float inverse rounds more)."""
    cams = [gi.camera_spline(2, f, 64) for f in (0, 5, 31)] + [gi.scene_light()]
    for cam in cams:
        for W, H in ((1920, 1080), (512, 512), (1024, 1024)):
            v = gi.view_from_camera(cam, W, H)
            rv, rp = r.camera_matrices(np.array(cam.pos, np.float32), cam.hor_angle, cam.vert_angle, cam.fovy,
                                       np.float32(W) / np.float32(H), cam.znear, cam.zfar)
            V, P = np.array(v.view, np.float32), np.array(v.proj, np.float32)
            ulp_v = np.spacing(np.abs(rv).max())
            ulp_p = np.abs(P - rp) / np.maximum(np.spacing(np.abs(rp)), np.spacing(np.float32(1e-30)))
            assert np.abs(V - rv).max() <= 4 * ulp_v, (cam.pos[:], np.abs(V - rv).max() / ulp_v)
            assert ulp_p.max() <= 1, ulp_p.max()


def test_march_equals_the_reference_shader_as_written(r, oracle, room512):
    """SSVGI/indirectLighting.frag exactly as the reference ships it (dirsCount =
    4, no step cap) on configuration 1's 512x512 room: the oracle's march is
    bit-identical on every pixel, with the same step count and the same mip level
    at every depth tap.  Beside it, the evaluation contract's distance to the
    shader as the reference would run it (glm float inverses per pixel) and both
    distances to the FP64 estimator."""
    s = room512
    view, gb = s["view"], s["gb"]
    got, trace = r.indirect(view.view, view.proj, 512, 512, s["lb"], s["db"], gb["normal"], gb["ndc"])
    with libm(oracle):
        ora, steps, otrace = oracle.march(_shader_view(r, view), 4, 0, s["lb"], s["db"], gb["normal"], gb["ndc"],
                                          lod_trace=True)
    assert np.array_equal(got, ora)
    assert np.array_equal(trace, otrace.reshape(trace.shape))
    assert np.array_equal(trace[:, 0], steps.ravel())
    contract, _, ctrace = oracle.march(view, 4, 0, s["lb"], s["db"], gb["normal"], gb["ndc"], lod_trace=True)
    assert np.array_equal(trace, ctrace.reshape(trace.shape))
    f64 = lambda lv: [x.astype(np.float64) for x in lv]
    d64, _ = oracle.march(view, 4, 0, f64(s["lb"]), f64(s["db"]), gb["normal"].astype(np.float64),
                          gb["ndc"].astype(np.float64), dtype=np.float64)
    l1 = lambda a, b: float(np.abs(a - b)[..., :3].sum() / np.abs(b[..., :3]).sum())
    rel = rel_err(contract[..., :3], got[..., :3], floor=1e-3 * np.abs(got[..., :3]).mean())
    print(f"512^2 R=4: contract vs reference shader frame L1 {l1(contract, got):.2e}, max rel {rel.max():.2e}; "
          f"vs FP64: reference shader {l1(got, d64):.2e}, contract {l1(contract, d64):.2e}")
    assert l1(contract, got) < 1e-4
    assert l1(contract, d64) < 2 * l1(got, d64) + 1e-5


def test_march_at_the_headline_directions(r, oracle, room1080):
    """The same shader with dirsCount = 16 (the headline's R; the step growth,
    step count and mip levels follow from it as written) at 1920x1080, on every
    17th row: bit-identical to the oracle, step counts and mip levels included."""
    s = room1080
    view, gb = s["view"], s["gb"]
    ys, xs = np.arange(3, 1080, 17), np.arange(1920)
    pix = np.stack(np.meshgrid(xs, ys), -1).reshape(-1, 2).astype(np.int32)
    got, trace = r.indirect(view.view, view.proj, 1920, 1080, s["lb"], s["db"], gb["normal"], gb["ndc"], dirs=16,
                            pixels=pix)
    with libm(oracle):
        ora, _, otrace = oracle.march(_shader_view(r, view), 16, 0, s["lb"], s["db"], gb["normal"], gb["ndc"],
                                      pixels=pix, lod_trace=True)
    assert np.array_equal(got, ora)
    assert np.array_equal(trace, otrace)
    contract, _, ctrace = oracle.march(view, 16, 0, s["lb"], s["db"], gb["normal"], gb["ndc"], pixels=pix,
                                       lod_trace=True)
    assert np.array_equal(trace, ctrace)
    rel = rel_err(contract[:, :3], got[:, :3], floor=1e-3 * np.abs(got[:, :3]).mean())
    print(f"1080p R=16 rows: contract vs reference shader max rel {rel.max():.2e}, mean {rel.mean():.2e}, "
          f"over 1e-3 {np.mean(rel > 1e-3) * 100:.3f}%")
    assert np.mean(rel > 1e-3) < 1e-2


def test_direct_gather_denoise_equal_the_reference_shaders(r, oracle, room512):
    """Common/directLighting.frag (with the shader's own inverses of both views),
    Common/finalGatherer.frag and Common/denoiser.frag (radius 0 and 2): bit-
    identical.  At radius 2 the reference's least-squares fit is singular on
    windows of constant depth and yields NaN there; the oracle reproduces every
    NaN at the same pixels."""
    s = room512
    view, light, gb = s["view"], s["light"], s["gb"]
    got = r.direct(view.view, view.proj, light.view, light.proj, gb["albedo"], gb["emissive"], gb["normal"],
                   gb["ndc"], s["sm"])
    with libm(oracle):
        ora = oracle.direct_light(_shader_view(r, view), _shader_view(r, light), gb, s["sm"])
    assert np.array_equal(got, ora)
    rng = np.random.default_rng(5)
    ind = rng.uniform(0.0, 1.0, (512, 512, 4)).astype(np.float32)
    assert np.array_equal(r.final_gather(s["direct"], s["lb"], gb["albedo"], ind),
                          oracle.final_gather(s["direct"], ind, gb["albedo"]))
    for radius in (0, 2):
        a = r.denoise(view.view, view.proj, ind, gb["moments"], gb["normal"], radius)
        b = oracle.denoise(ind, gb["moments"], radius)
        assert np.array_equal(np.isnan(a), np.isnan(b))
        ok = ~np.isnan(a)
        assert np.array_equal(a[ok], b[ok])
        if radius == 2:
            print(f"denoiser radius 2: {np.isnan(a[..., 0]).mean() * 100:.2f}% of pixels NaN in the reference")
