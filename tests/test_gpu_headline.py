"""The benchmark's headline configuration held to the per-pixel bar, and the
texture units' sampler arithmetic that its march precision relies on.

* The texture-unit sampler: fetches through the library's pyramid textures
  (gi_texture_sample, the fetch GI_MARCH_TEXTURE makes per step) against the
  oracle's restatement of the units' fixed point (oracle/sampler.h
  texture_lod_unit), at random coordinates -- inside, at and beyond the edges --
  and random levels.
* The headline frame: 1920x1080, R = 16 directions, step cap 64, two bounces
  (the second re-lights the first one's recorded march), 5x5 bilateral, a seeded
  room of 64 boxes and 16 spheres -- the workload bench.py times -- as one whole
  frame against the oracle's frame (SSVGIRenderer.h:207-342 restated), in every
  march precision:
    exact    bit-identical to the fp32 oracle (>= 99.9 % of values; the rest
             within 1e-3),
    fast     within 1e-3 relative per value of the fp32 oracle,
    texture  within 1e-3 relative per value of the oracle with the texture-unit
             sampler on the same taps (depth taps of both bounces, light taps of
             the first; the second bounce re-lights with software taps).
  Relative error per value is |got - ref| / max(|ref|, 1e-3 * mean |ref|) over
  the lit image's rgb.  Each precision's error against the FP64 re-evaluation of
  the same estimator is printed beside it.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

RADIANCE_RTOL = 1e-3


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("channels,src_channels", [(1, 2), (4, 4)])
def test_texture_unit_sampler_matches_oracle(gi, oracle, cuda, channels, src_channels):
    """Every fetch equals the oracle's fixed-point restatement to fp32 rounding
    (the units' accumulation order is not observable: <= 1e-6 relative), and the
    restatement is far from the exact sampler (it is the 8-bit weights that
    matter, not rounding)."""
    torch = cuda
    rng = np.random.default_rng(31 + channels)
    W, H = 640, 360
    L = gi.mip_level_count(W, H, 10)
    base = rng.uniform(0.2, 3.0, (H, W, src_channels)).astype(np.float32)
    levels = oracle.mip_chain(base, L)
    n = 100_000
    coords = rng.uniform(-0.1, 1.1, (n, 2)).astype(np.float32)
    lods = rng.uniform(-0.5, L + 0.5, n).astype(np.float32)
    got = torch.empty((n, channels), dtype=torch.float32, device="cuda")
    gi.texture_sample([dev(torch, x) for x in levels], channels, dev(torch, coords), dev(torch, lods), got)
    torch.cuda.synchronize()
    got = host(got)
    ref = oracle.texture_unit(levels, coords, lods, channels)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3)
    same = float(np.mean(got == ref))
    # The exact (Vulkan-formula) sampler at the same points, for scale.
    exact = oracle.texture_unit_exact(levels, coords, lods, channels)
    far = np.abs(exact - ref).max()
    print(f"texture units vs oracle ({channels} ch): max rel {rel.max():.2e}, bit-identical {same * 100:.2f}%; "
          f"exact sampler differs by up to {far:.2e}")
    assert rel.max() <= 1e-6
    assert same >= 0.98
    assert far > 1e-3


def _headline_inputs(gi, oracle, W=1920, H=1080, seed=2000, spline=2, frame=5):
    prims = gi.scene_generate(seed, 64, 16)
    view = gi.view_from_camera(gi.camera_spline(spline, frame, 64), W, H)
    light = gi.view_from_camera(gi.scene_light(), 1024, 1024)
    gb = oracle.gbuffer(view, prims)
    direct = oracle.direct_light(view, light, gb, oracle.shadow_map(light, prims))
    return view, gb, direct


def _gpu_frame(gi, torch, view, gb, direct, precision):
    ins = [dev(torch, x) for x in (gb["albedo"], gb["normal"], gb["moments"], gb["ndc"], direct)]
    r = gi.Renderer(view.width, view.height, dirs=16, step_cap=64, bounces=2, bilateral=True, precision=precision)
    lit = torch.empty((view.height, view.width, 4), dtype=torch.float32, device="cuda")
    r.render(view, *ins, lit)
    torch.cuda.synchronize()
    r.close()
    return host(lit)[..., :3]


def test_headline_frame_1080p_two_bounces(gi, oracle, cuda):
    torch = cuda
    view, gb, direct = _headline_inputs(gi, oracle)
    ref = oracle.render_frame(view, gb, direct, 16, 64, bounces=2)["lit"][..., :3]
    ref_tex = oracle.render_frame(view, gb, direct, 16, 64, bounces=2, texture=True)["lit"][..., :3]
    gb64 = {k: v.astype(np.float64) for k, v in gb.items()}
    ref64 = oracle.render_frame(view, gb64, direct.astype(np.float64), 16, 64, bounces=2)["lit"][..., :3]
    floor = 1e-3 * float(np.abs(ref).mean())

    def fp64_err(x):
        return float(np.abs(x - ref64).sum() / np.abs(ref64).sum())

    results = {}
    for name, prec, oracle_frame in (("exact", gi.GI_MARCH_EXACT, ref), ("fast", gi.GI_MARCH_FAST, ref),
                                     ("texture", gi.GI_MARCH_TEXTURE, ref_tex)):
        got = _gpu_frame(gi, torch, view, gb, direct, prec)
        rel = rel_err(got, oracle_frame, floor=floor)
        results[name] = (got, rel)
        print(f"1920x1080 R=16 cap 64, 2 bounces, {name}: max rel {rel.max():.2e} vs its oracle frame, "
              f"bit-identical {np.mean(got == oracle_frame) * 100:.3f}%, over 1e-4 {np.mean(rel > 1e-4) * 100:.4f}%; "
              f"frame rel L1 vs FP64 {fp64_err(got):.3e} (fp32 oracle {fp64_err(ref):.3e})")
    got, rel = results["exact"]
    assert np.mean(got == ref) >= 0.999
    assert rel.max() <= RADIANCE_RTOL
    assert results["fast"][1].max() <= RADIANCE_RTOL
    assert results["texture"][1].max() <= RADIANCE_RTOL
    for got, _ in results.values():
        assert np.isfinite(got).all()
