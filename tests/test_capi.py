"""The C ABI without a GPU: the library loads, exports every symbol that
include/legit_gi.h declares, and its host-side logic (geometry, views, the
procedural scene, argument validation) behaves."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "legit_gi.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^GI_API\s+[\w\s\*]+?\b(gi_\w+)\s*\(", text, flags=re.M)))


def test_every_declared_symbol_is_exported(gi):
    L = gi.lib()
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) <= set(gi.exported_symbols()) | set(syms)
    out = subprocess.run(["nm", "-D", "--defined-only", str(gi.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (gi_\w+)", out))
    assert set(syms) <= exported
    # Only the ABI is exported (everything else is hidden).
    assert all(s in syms for s in exported), sorted(exported - set(syms))


def test_status_strings(gi):
    L = gi.lib()
    assert L.gi_abi_version() == 1
    assert L.gi_status_string(0) == b"ok"
    assert L.gi_status_string(1) == b"invalid argument"
    assert L.gi_status_string(99) == b"unknown status"


def test_invalid_arguments_are_reported_not_thrown(gi):
    L = gi.lib()
    null = C.c_void_p(0)
    assert L.gi_build_mips(null, 64, 64, 4, 2, 0, null) == 1
    assert b"bad image" in L.gi_last_error()
    lv = (C.c_void_p * 2)(16, 32)
    assert L.gi_build_mips(lv, 64, 64, 3, 2, 0, null) == 1          # 3 channels
    assert L.gi_build_mips(lv, 64, 64, 4, 8, 0, null) == 1          # more levels than 64x64 has
    assert L.gi_build_mips(lv, 64, 64, 4, 2, 7, null) == 1          # bad filter
    assert L.gi_blur(null, null, 4, 4, 4, 2, null) == 1
    assert L.gi_deinterleave(C.c_void_p(16), C.c_void_p(32), 10, 8, 4, 4, 4, null) == 1  # 10 % 4 != 0
    assert b"multiple of the grid" in L.gi_last_error()
    assert L.gi_interleave(C.c_void_p(16), C.c_void_p(16), 8, 8, 4, 4, 4, null) == 1     # aliased
    v = gi.GiView()
    v.width, v.height = 64, 64
    p = gi.GiMarchParams(0, 64, 4)
    levels = (C.c_void_p * 1)(16)
    assert L.gi_march(C.byref(v), C.byref(p), levels, levels, 1, C.c_void_p(16), C.c_void_p(16),
                      C.c_void_p(16), null) == 1                          # dirs = 0
    p = gi.GiMarchParams(4, 64, 4)
    assert L.gi_march(C.byref(v), C.byref(p), levels, levels, 1, C.c_void_p(16), C.c_void_p(16),
                      C.c_void_p(24), null) == 1                          # unaligned output
    assert b"unaligned" in L.gi_last_error()
    fp = gi.GiFrameParams()
    fp.march = gi.GiMarchParams(16, 64, 4)
    fp.bounces, fp.bilateral, fp.denoise_radius, fp.mip_levels = 0, 1, 0, 10
    h = C.c_void_p()
    assert L.gi_renderer_create(64, 64, C.byref(fp), C.byref(h)) == 1    # zero bounces
    assert L.gi_renderer_render(null, None, None, null, null, null) == 1
    fp.bounces = 2
    fp.march = gi.GiMarchParams(16, 64, 4, 0, 3)
    assert L.gi_renderer_create(64, 64, C.byref(fp), C.byref(h)) == 1    # no precision 3
    assert b"unknown precision" in L.gi_last_error()
    p = gi.GiMarchParams(4, 64, 4, 0, 3)
    assert L.gi_march(C.byref(v), C.byref(p), levels, levels, 1, C.c_void_p(16), C.c_void_p(16),
                      C.c_void_p(32), null) == 1
    assert b"unknown precision" in L.gi_last_error()


def test_precision_constants_match_the_header(gi):
    """The march precisions the Python binding names are the header's values."""
    text = HEADER.read_text()
    defs = dict(re.findall(r"^#define (GI_MARCH_\w+) (\d+)", text, flags=re.M))
    assert defs == {"GI_MARCH_EXACT": "0", "GI_MARCH_FAST": "1", "GI_MARCH_TEXTURE": "2"}
    for name, value in defs.items():
        assert getattr(gi, name) == int(value), name
    losses = dict(re.findall(r"^#define (GI_MLP_LOSS_\w+) (\d+)", text, flags=re.M))
    assert losses == {"GI_MLP_LOSS_SQUARED": "0", "GI_MLP_LOSS_ABSOLUTE": "1"}
    for name, value in losses.items():
        assert getattr(gi, name) == int(value), name


def test_scene_is_seeded_and_bounded(gi):
    a = bytes(gi.scene_generate(2000, 64, 16))
    b = bytes(gi.scene_generate(2000, 64, 16))
    c = bytes(gi.scene_generate(2001, 64, 16))
    assert a == b and a != c
    prims = gi.scene_generate(2000, 64, 16)
    assert len(prims) == 81 and prims[0].kind == gi.GI_PRIM_ROOM
    for p in prims[1:65]:
        assert p.kind == gi.GI_PRIM_BOX
        for k in range(3):
            s = p.b[k] - p.a[k]
            assert 0.05 - 1e-6 <= s <= 0.3 + 1e-6 and p.a[k] >= 0.0 and p.b[k] <= 1.0
        assert p.b[1] <= 0.85 + 1e-6
        for c in range(4):
            q = round(p.albedo[c] * 255)
            assert abs(p.albedo[c] * 255 - q) < 1e-3 and 51 <= q <= 230
    for p in prims[65:]:
        assert p.kind == gi.GI_PRIM_SPHERE and 0.05 - 1e-6 <= p.b[0] <= 0.2 + 1e-6


def test_views_are_consistent(gi):
    cam = gi.camera_spline(7, 11, 64)
    v = gi.view_from_camera(cam, 1920, 1080)
    m = lambda a: np.array(list(a), np.float64).reshape(4, 4).T  # column-major -> row-major
    vp, ivp = m(v.view_proj), m(v.inv_view_proj)
    assert np.allclose(vp @ ivp, np.eye(4), atol=1e-4)
    assert np.allclose(m(v.proj) @ m(v.view), vp, rtol=1e-5, atol=1e-6)
    # The camera position is the translation column of the inverse view.
    iv = m(v.inv_view)
    assert np.allclose(iv[:3, 3], list(cam.pos), atol=1e-6)
    # A point straight ahead of the camera projects to the screen centre with depth in (0, 1).
    fwd = np.array([np.cos(cam.vert_angle) * np.sin(cam.hor_angle), -np.sin(cam.vert_angle),
                    np.cos(cam.vert_angle) * np.cos(cam.hor_angle)])
    p = vp @ np.append(np.array(cam.pos) + 0.5 * fwd, 1.0)
    ndc = p[:3] / p[3]
    assert abs(ndc[0]) < 1e-4 and abs(ndc[1]) < 1e-4 and 0.0 < ndc[2] < 1.0
    # Spline is closed: frame 64 == frame 0.
    a, b = gi.camera_spline(7, 0, 64), gi.camera_spline(7, 64, 64)
    assert list(a.pos) == list(b.pos)


def test_render_graph_shim_compiles(tmp_path):
    """Host code written against the reference's AddPass/RenderPassDesc surface compiles."""
    src = tmp_path / "use_shim.cpp"
    src.write_text(r'''
#include "legit_render_graph.h"
void Record(legit::RenderGraph* rg, legit::ShaderMemoryPool* pool, legit::MippedProxy& light,
            legit::MippedProxy& blurred, legit::UnmippedProxy& a, legit::UnmippedProxy& b) {
  legit::MipBuilder mipBuilder;
  legit::BlurBuilder blurBuilder;
  legit::InterleaveBuilder interleaveBuilder;
  mipBuilder.BuildMips(rg, pool, light);
  for (uint32_t mip = 0; mip < light.mipImageViewProxies.size(); mip++)
    blurBuilder.ApplyBlur(rg, pool, light.mipImageViewProxies[mip]->Id(), blurred.mipImageViewProxies[mip]->Id(),
                          mip == 0 ? 0 : 2);
  interleaveBuilder.Deinterleave(rg, pool, a.imageViewProxy->Id(), b.imageViewProxy->Id(), legit::uvec2(4, 4));
  rg->AddPass(legit::RenderGraph::RenderPassDesc()
                  .SetColorAttachments({b.imageViewProxy->Id()})
                  .SetInputImages({a.imageViewProxy->Id()})
                  .SetRenderAreaExtent(legit::Extent2D(64, 64))
                  .SetProfilerInfo(legit::Colors::sunFlower, "Custom")
                  .SetRecordFunc([](legit::RenderGraph::RenderPassContext ctx) { (void)ctx.GetCommandBuffer(); }));
}
''')
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{ROOT / 'legitengine_gb300' / 'csrc'}",
                        f"-I{ROOT / 'include'}", f"-I{cuda_inc}", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_march_layouts_are_recorded_and_validated(gi):
    """gi_march_set_layout / gi_march_tuned_layout (host-side table): a layout is
    CTA rows with 32 x dirs rays per warp (one thread per pixel) or 4 rows with
    32 x ceil(dirs / 4) (the direction split, 4 to 32 directions); it is kept per
    shape and precision; anything else is refused with GI_ERR_INVALID_ARGUMENT."""
    W, H, cap = 977, 311, 40
    assert gi.march_tuned_layout(W, H, 12, 0, cap, 1) == (0, 0)
    gi.march_set_layout(W, H, 12, 0, cap, 1, 8, 32 * 12)
    assert gi.march_tuned_layout(W, H, 12, 0, cap, 1) == (8, 384)
    assert gi.march_tuned_layout(W, H, 12, 0, cap, 2) == (0, 0)  # another precision
    gi.march_set_layout(W, H, 12, 0, cap, 2, 4, 32 * 3)
    assert gi.march_tuned_layout(W, H, 12, 0, cap, 2) == (4, 96)
    assert gi.march_tuned_layout(W, H, 12, 12, cap, 2) == (4, 96)  # step_dirs 0 means dirs
    gi.march_set_layout(W, H, 5, 0, cap, 0, 4, 64)  # 5 directions: a thread marches 2 of them
    assert gi.march_tuned_layout(W, H, 5, 0, cap, 0) == (4, 64)
    assert gi.lib().gi_march_tuned_rows(W, H, 5, 0, cap) == 4
    for bad in ((W, H, 12, 0, cap, 1, 3, 384), (W, H, 12, 0, cap, 1, 2, 96), (W, H, 12, 0, cap, 1, 4, 100),
                (W, H, 2, 0, cap, 1, 4, 32), (W, H, 40, 0, cap, 1, 4, 320), (W, H, 12, 0, cap, 3, 4, 384),
                (0, H, 12, 0, cap, 1, 4, 384)):
        with pytest.raises(gi.GiError) as e:
            gi.march_set_layout(*bad)
        assert e.value.status == gi.GI_ERR_INVALID_ARGUMENT
