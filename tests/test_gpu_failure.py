"""Failure paths, made to happen without faulting the GPU.

* A bounded wait that runs out: the tensor-core reconstruction's completion
  waits give up after a bound; the test hook gi_debug_tensor_core_wait_limit
  shortens the first wait of each tile group so that it runs out.  The launch
  must return, count the error (gi_mlp_tensor_core_errors), leave the context
  usable, and the next normal launch must give the normal result bit for bit.
* Device allocations that fail: the test hook gi_debug_fail_allocations makes
  the library's Nth allocation fail.  Creating and rendering with a renderer,
  for every N until both succeed, must fail with GI_ERR_OUT_OF_MEMORY and
  leak nothing (gi_debug_live_allocations back to where it started), and a
  renderer whose frame failed must render the next frame correctly.
"""
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


@pytest.fixture(scope="module")
def frame(gi, oracle, cuda):
    torch = cuda
    W, H = 256, 144
    prims = gi.scene_generate(1000, 16, 0)
    view = gi.view_from_camera(gi.camera_spline(1, 3, 64), W, H)
    light = gi.view_from_camera(gi.scene_light(), 256, 256)
    gb = oracle.gbuffer(view, prims)
    direct = oracle.direct_light(view, light, gb, oracle.shadow_map(light, prims))
    ins = [dev(torch, x) for x in (gb["albedo"], gb["normal"], gb["moments"], gb["ndc"], direct)]
    return view, ins


def test_tensor_core_wait_that_runs_out(gi, cuda, frame):
    torch = cuda
    view, (albedo, normal, moments, ndc, direct) = frame
    W, H = view.width, view.height
    few = gi.alloc_pyramid(W, H, 4, 5)
    gi.march(view, gi.GiMarchParams(2, 32, 4, 32, gi.GI_MARCH_EXACT), *_pyramids(gi, torch, W, H, direct, moments),
             normal, ndc, few[0])
    gi.build_mips(few, 4)
    filt = torch.empty_like(few[0])
    gi.bilateral(few[0], moments, normal, filt)
    L = gi.mip_level_count(W, H, 10)
    db = _pyramids(gi, torch, W, H, direct, moments)[1]
    net = gi.Mlp(seed=3)

    def run():
        out = torch.full((H, W, 4), float("nan"), dtype=torch.float32, device="cuda")
        net.reconstruct(moments, normal, albedo, direct, [few[0], few[2], few[4]], filt, db[2], out)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    good = run()
    e0 = gi.tensor_core_errors()
    try:
        gi.debug_tensor_core_wait_limit(1)
        broken = run()  # the launch returns; its groups stop at their first wait
        e1 = gi.tensor_core_errors()
    finally:
        gi.debug_tensor_core_wait_limit(0)
    assert e1 > e0, "no wait ran out"
    assert np.isnan(broken).any(), "every tile was written although its group stopped"
    again = run()
    assert np.array_equal(again, good)
    assert gi.tensor_core_errors() == e1
    assert L >= 5


def _pyramids(gi, torch, W, H, direct, moments):
    L = gi.mip_level_count(W, H, 10)
    ll, dl = gi.alloc_pyramid(W, H, 4, L), gi.alloc_pyramid(W, H, 2, L)
    ll[0].copy_(direct)
    dl[0].copy_(moments)
    gi.build_mips(ll, 4)
    gi.build_mips(dl, 2)
    lb = [ll[0]] + gi.alloc_pyramid(W, H, 4, L)[1:]
    db = [dl[0]] + gi.alloc_pyramid(W, H, 2, L)[1:]
    gi.blur_pyramid(ll, lb)
    gi.blur_pyramid(dl, db)
    return lb, db


@pytest.mark.parametrize("precision", [0, 2])
def test_failed_allocations_leak_nothing(gi, cuda, frame, precision):
    torch = cuda
    view, ins = frame
    W, H = view.width, view.height
    kw = dict(dirs=8, step_cap=32, bounces=2, bilateral=True, precision=precision)
    lit = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    ref = gi.Renderer(W, H, **kw)
    ref.render(view, *ins, lit)
    torch.cuda.synchronize()
    expected = lit.cpu().numpy()
    ref.close()
    # Objects of earlier tests free their device memory from finalizers: collect
    # them now and keep the collector off while the live count is compared.
    gc.collect()
    gc.disable()
    try:
        _inject_until_done(gi, torch, view, ins, lit, kw, expected, precision)
    finally:
        gc.enable()


def _inject_until_done(gi, torch, view, ins, lit, kw, expected, precision):
    W, H = view.width, view.height
    base = gi.debug_live_allocations()
    failures, done = 0, False
    for after in range(200):
        r = None
        try:
            gi.debug_fail_allocations(after)
            r = gi.Renderer(W, H, **kw)
            r.render(view, *ins, lit)
            torch.cuda.synchronize()
            done = True
        except gi.GiError as e:
            assert e.status == gi.GI_ERR_OUT_OF_MEMORY, e
            failures += 1
            if r is not None:  # created, its first frame failed: the next frame renders
                gi.debug_fail_allocations(-1)
                r.render(view, *ins, lit)
                torch.cuda.synchronize()
                assert np.array_equal(lit.cpu().numpy(), expected)
        finally:
            gi.debug_fail_allocations(-1)
            if r is not None:
                r.close()
        live = gi.debug_live_allocations()
        assert live == base, f"allocation {after}: {live} live allocations, {base} before"
        if done:
            break
    assert done and failures >= 3
    assert np.array_equal(lit.cpu().numpy(), expected)
    print(f"renderer (precision {precision}): {failures} injected failure points, none leaked")
