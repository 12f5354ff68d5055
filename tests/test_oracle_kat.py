"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests or golden images, so the oracle is pinned by
tables derived from the reference's formulas: the Hammersley sequence
(indirectLighting.frag:102-112), the interleave maps (deinterleave.frag,
interleave.frag), the mip geometry (MipBuilder.h:146-152), the per-direction
step counts (:212), and the horizon integral (:44-49)."""
import math

import numpy as np
import pytest

from conftest import rel_err


def test_hammersley_table(oracle):
    # x = i / 16; y = bit-reversed radical inverse of i.
    assert oracle.hammersley(0, 16) == (0.0, 0.0)
    assert oracle.hammersley(1, 16) == (0.0625, 0.5)
    assert oracle.hammersley(2, 16) == (0.125, 0.25)
    assert oracle.hammersley(3, 16) == (0.1875, 0.75)
    assert oracle.hammersley(15, 16) == (0.9375, 0.9375)
    for i in range(16):
        rev = int(format(i, "032b")[::-1], 2)
        assert oracle.hammersley(i, 16)[1] == np.float32(rev) / np.float32(4294967296.0)


@pytest.mark.parametrize("w,h", [(512, 512), (1920, 1080), (640, 480), (16, 8)])
def test_interleave_maps_are_inverse_bijections(oracle, w, h):
    d = oracle.deinterleave_map(w, h)
    i = oracle.interleave_map(w, h)
    assert np.array_equal(np.sort(d), np.arange(w * h))
    assert np.array_equal(d[i], np.arange(w * h))
    assert np.array_equal(i[d], np.arange(w * h))


def test_deinterleave_layout_known_answer(oracle):
    # 8x4 image, grid 4x4 -> sub-images of 2x1; sub-image (kx, ky) holds pixels (kx + 4i, ky).
    w, h = 8, 4
    d = oracle.deinterleave_map(w, h)
    img = np.arange(w * h).reshape(h, w)
    dst = img.ravel()[d].reshape(h, w)
    assert dst[0].tolist() == [0, 4, 1, 5, 2, 6, 3, 7]
    assert dst[1].tolist() == [8, 12, 9, 13, 10, 14, 11, 15]


@pytest.mark.parametrize("w,h,levels,last", [
    (1920, 1080, 10, (3, 2)), (512, 512, 10, (1, 1)), (640, 480, 9, (2, 1)), (256, 256, 9, (1, 1)),
    (1280, 720, 10, (2, 1)), (2048, 1152, 10, (4, 2)), (3840, 2160, 10, (7, 4)),
])
def test_mip_geometry(gi, oracle, w, h, levels, last):
    assert gi.mip_level_count(w, h, 10) == levels
    assert oracle.mip_level_count(w, h, 10) == levels
    assert gi.mip_level_size(w, h, levels - 1) == last
    sizes = [(w, h)]
    for _ in range(1, levels):
        sizes.append((sizes[-1][0] // 2, sizes[-1][1] // 2))
    assert all(gi.mip_level_size(w, h, k) == sizes[k] for k in range(levels))


def test_step_count_known_answers(oracle):
    # 1920x1080, R = 4: 7 steps from the centre along +x, 8 from a corner along the diagonal.
    assert oracle.iterations(1920, 1080, 4, 960.5, 540.5, 1.0, 0.0) == 7
    assert oracle.iterations(1920, 1080, 4, 960.5, 540.5, 0.0, 1.0) == 6
    d = 1.0 / math.sqrt(1920 ** 2 + 1080 ** 2)
    assert oracle.iterations(1920, 1080, 4, 0.5, 0.5, 1920 * d, 1080 * d) == 8
    # More directions take denser steps: R = 16 from the centre along +x.
    assert oracle.iterations(1920, 1080, 16, 960.5, 540.5, 1.0, 0.0) == 19
    assert oracle.iterations(1920, 1080, 16, 960.5, 540.5, 1.0, 0.0, cap=12) == 12


def test_horizon_contribution_is_the_cosine_weighted_slice_integral(oracle):
    """HC(a, b) = integral_a^b (n . (e cos t + g sin t)) sin t dt  (indirectLighting.frag:44-49)."""
    from scipy.integrate import quad
    rng = np.random.default_rng(5)
    for _ in range(20):
        e, g = rng.normal(size=3), rng.normal(size=3)
        n = rng.normal(size=3)
        a, b = np.sort(rng.uniform(-1.5, 1.5, size=2))
        ref = quad(lambda t: np.dot(n, e * np.cos(t) + g * np.sin(t)) * np.sin(t), a, b)[0]
        hc = oracle.horizon_contribution(e, g, n, a, b)
        assert abs(hc - ref) < 1e-9


def test_mip_and_blur_known_answers(oracle):
    img = np.arange(4 * 4 * 1, dtype=np.float32).reshape(4, 4, 1)
    m = oracle.mip_level(img, 0)
    assert m[..., 0].tolist() == [[2.5, 4.5], [10.5, 12.5]]
    dm = np.stack([img[..., 0], img[..., 0] + 1.0, np.ones((4, 4), np.float32), np.zeros((4, 4), np.float32)],
                  axis=-1)
    mm = oracle.mip_level(np.ascontiguousarray(dm), 1)
    assert mm[0, 0, 0] == 0.0 and mm[0, 0, 1] == 6.0 and mm[0, 0, 3] == 0.0
    # mass: sum((y - x) * z) / (max - min) / 4 = 4 / 6 / 4
    assert mm[0, 0, 2] == np.float32(np.float32(4.0) / np.float32(6.0) / np.float32(4.0))
    # radius-2 box blur at (0, 0): taps x, y in [-2, 2) clamped -> texels (0..1, 0..1) weighted 9, 3, 3, 1.
    b = oracle.blur(img, 2)
    assert b[0, 0, 0] == np.float32((9 * 0 + 3 * 1 + 3 * 4 + 1 * 5) / 16.0)
    assert np.array_equal(oracle.blur(img, 0), img)


def test_fp32_oracle_tracks_fp64(oracle, scene_small):
    """The fp32 restatement stays within 1e-3 of the FP64 re-evaluation of the same estimator."""
    s = scene_small
    gb64 = {k: v.astype(np.float64) for k, v in s["gb"].items()}
    o32 = oracle.render_frame(s["view"], s["gb"], s["direct"], 8, 32, bounces=1)
    o64 = oracle.render_frame(s["view"], gb64, s["direct"].astype(np.float64), 8, 32, bounces=1)
    e = rel_err(o32["lit"][..., :3], o64["lit"][..., :3], floor=1e-2)
    assert e.max() < 1e-3, e.max()


@pytest.mark.parametrize("name", ["reconstructor_1dir.bin", "reconstructor_2dir.bin"])
def test_committed_reconstructor_weights_are_finite(name):
    """The shipped checkpoints: GIMLP001 header, parameter count, CRC, finite weights."""
    import zlib
    from pathlib import Path
    raw = (Path(__file__).resolve().parents[1] / "legitengine_gb300" / "data" / name).read_bytes()
    assert raw[:8] == b"GIMLP001"
    n = int(np.frombuffer(raw[8:12], np.uint32)[0])
    assert n == 10627 and len(raw) == 16 + n * 12 + 4
    assert zlib.crc32(raw[:-4]) == int(np.frombuffer(raw[-4:], np.uint32)[0])
    assert np.isfinite(np.frombuffer(raw[16:16 + n * 4], np.float32)).all()


def test_golden_known_answers(gi, oracle):
    """The oracle and the library against tests/golden/kat.json, which
    tests/golden/make_golden.py derives from the reference's formulas in plain
    Python (Hammersley table, mip geometry of every configured resolution, the 4x4
    deinterleave map, per-direction step counts)."""
    import json
    from pathlib import Path
    kat = json.loads((Path(__file__).resolve().parent / "golden" / "kat.json").read_text())
    for i, (x, y) in enumerate(kat["hammersley_16"]):
        assert oracle.hammersley(i, 16) == (np.float32(x), np.float32(y)), i
    for key, sizes in kat["mip_geometry"].items():
        w, h = map(int, key.split("x"))
        assert gi.mip_level_count(w, h, 10) == len(sizes) == oracle.mip_level_count(w, h, 10), key
        assert [list(gi.mip_level_size(w, h, k)) for k in range(len(sizes))] == sizes, key
    assert oracle.deinterleave_map(8, 8).tolist() == kat["deinterleave_8x8_source"]
    for c in kat["step_counts"]:
        assert oracle.iterations(c["w"], c["h"], c["R"], c["c"][0], c["c"][1], c["d"][0], c["d"][1]) == c["n"], c


def test_texture_unit_sampler_reproduces_measured_weights(oracle):
    """oracle/sampler.h texture_lod_unit against texel weights the GPU's texture
    units returned (tests/golden/texture_unit_weights.npz, measured through the
    library's texture path by tests/golden/make_texture_weights.py): every one of
    the eight trilinear weights of 3000 random points, exactly."""
    from pathlib import Path
    path = Path(__file__).resolve().parent / "golden" / "texture_unit_weights.npz"
    f = np.load(path)
    W, H, L = (int(x) for x in f["size"])
    coords, lods, weights = f["coords"], f["lods"], f["weights"]
    for lev in range(L):
        for p in range(4):
            levels = []
            for k in range(L):
                a = np.zeros((H >> k, W >> k, 1), np.float32)
                if k == lev:
                    a[(p >> 1)::2, (p & 1)::2, 0] = 1.0
                levels.append(a)
            got = oracle.texture_unit(levels, coords, lods, 1)[:, 0] * 256.0
            assert np.array_equal(got, weights[lev, p].astype(np.float32)), (lev, p)
    # The exact sampler (fp32 Vulkan formulas) does not: the weights are the units' own.
    ex = oracle.texture_unit_exact([np.ones((H >> k, W >> k, 1), np.float32) * (k == 0) for k in range(L)],
                                   coords, lods, 1)[:, 0] * 256.0
    assert not np.array_equal(ex, weights[0].sum(0).astype(np.float32))


def test_oracle_scenes_and_views_equal_the_library(gi, oracle):
    """The oracle's own restatement of the benchmark's frames (go_scene_generate,
    go_scene_light, go_camera_spline, go_view_from_camera), which the CPU reference
    arm uses instead of the library: scenes, light and cameras byte-identical;
    view matrices within one float ulp of each matrix's largest entry (the oracle
    inverts by the adjugate, the library by elimination)."""
    for seed, boxes, spheres in ((2000, 64, 16), (1000, 16, 0), (5003, 256, 64)):
        assert bytes(gi.scene_generate(seed, boxes, spheres)) == bytes(oracle.scene_generate(seed, boxes, spheres))
    assert bytes(gi.scene_light()) == bytes(oracle.scene_light())
    prims = gi.scene_generate(2000, 64, 16)
    for f in range(0, 64, 3):
        for pr in (None, prims):
            c = gi.camera_spline(2, f, 64, pr)
            assert bytes(c) == bytes(oracle.camera_spline(2, f, 64, pr))
            for w, h in ((1920, 1080), (512, 512)):
                a, b = gi.view_from_camera(c, w, h), oracle.view_from_camera(c, w, h)
                for field in ("view", "proj", "view_proj", "inv_view", "inv_proj", "inv_view_proj"):
                    x = np.array(getattr(a, field), np.float32)
                    y = np.array(getattr(b, field), np.float32)
                    assert np.abs(x - y).max() <= np.spacing(np.abs(x).max()), (f, field)
