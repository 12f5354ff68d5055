"""Python binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker of the CUDA path; the shipped library never imports it.  Arrays are
numpy, images (H, W, C).  dtype float32 gives the fp32 parity oracle, float64
the FP64 error reference.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from legitengine_gb300.gi import GiCamera, GiPrim, GiView  # noqa: E402  (struct layouts of the public ABI)

from . import build_oracle  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(str(path))
        _lib = L
        L.go_threads.restype = C.c_int
        for n in ("go_logf", "go_log2f", "go_expf", "go_exp2f", "go_sinf", "go_cosf"):
            getattr(L, n).restype = C.c_float
            getattr(L, n).argtypes = [C.c_float]
        for n in ("go_powf", "go_atan2f"):
            getattr(L, n).restype = C.c_float
            getattr(L, n).argtypes = [C.c_float, C.c_float]
        L.go_mip_level_count.restype = C.c_int
        L.go_iterations_f32.restype = C.c_int
        L.go_iterations_f32.argtypes = [C.c_int] * 4 + [C.c_float] * 4
        L.go_horizon_contribution_f64.restype = C.c_double
        L.go_horizon_contribution_f64.argtypes = [C.c_void_p] * 3 + [C.c_double] * 2
    return _lib


def scene_generate(seed: int, num_boxes: int, num_spheres: int):
    """The seeded room (go_scene_generate), a GiPrim array: the library's scene of
    the same seed, built without the library."""
    n = 1 + num_boxes + num_spheres
    arr = (GiPrim * n)()
    cnt = C.c_int()
    if lib().go_scene_generate(C.c_uint64(seed), num_boxes, num_spheres, arr, n, C.byref(cnt)) != 0:
        raise ValueError("go_scene_generate: bad arguments")
    return arr


def scene_light():
    c = GiCamera()
    lib().go_scene_light(C.byref(c))
    return c


def camera_spline(seed: int, frame: int, num_frames: int, prims=None):
    c = GiCamera()
    lib().go_camera_spline(C.c_uint64(seed), prims, 0 if prims is None else len(prims), frame, num_frames,
                           C.byref(c))
    return c


def view_from_camera(cam, width: int, height: int):
    v = GiView()
    if lib().go_view_from_camera(C.byref(cam), width, height, C.byref(v)) != 0:
        raise ValueError("go_view_from_camera: singular camera or projection")
    return v


def threads() -> int:
    return lib().go_threads()


def set_libm(on: bool):
    """fp32 transcendentals and division from the C library instead of the
    evaluation contract (test of the restatement against oracle/_ref only)."""
    lib().go_set_libm(int(on))


def set_threads(n: int):
    lib().go_set_threads(int(n))


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def _sfx(dtype) -> str:
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


MATH_FN = {"log": 0, "log2": 1, "exp": 2, "exp2": 3, "pow": 4, "atan2": 5, "sin": 6, "cos": 7}


def math_batch(fn: str, a, b=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(np.zeros_like(a) if b is None else b, dtype=np.float32)
    out = np.empty_like(a)
    lib().go_math_batch(MATH_FN[fn], _p(a), _p(b), _p(out), C.c_int(a.size))
    return out


def hammersley(i: int, n: int) -> tuple[float, float]:
    out = np.zeros(2, np.float32)
    lib().go_hammersley(i, n, _p(out))
    return float(out[0]), float(out[1])


def iterations(W: int, H: int, R: int, cx: float, cy: float, dx: float, dy: float, cap: int = 0) -> int:
    """Steps of one direction (indirectLighting.frag:201-212), fp32."""
    return lib().go_iterations_f32(W, H, R, cap, cx, cy, dx, dy)


def horizon_contribution(ed, et, n, mn: float, mx: float) -> float:
    """ComputeHorizonContribution (indirectLighting.frag:44-49) in double."""
    a = [np.ascontiguousarray(v, np.float64) for v in (ed, et, n)]
    return lib().go_horizon_contribution_f64(_p(a[0]), _p(a[1]), _p(a[2]), mn, mx)


def mip_level_count(w: int, h: int, req: int = 10) -> int:
    return lib().go_mip_level_count(w, h, req)


def mip_level(src: np.ndarray, filter: int = 0) -> np.ndarray:
    sh, sw, ch = src.shape
    dst = np.zeros((sh // 2, sw // 2, ch), src.dtype)
    getattr(lib(), "go_mip_level_" + _sfx(src.dtype))(_p(src), sw, sh, ch, _p(dst), sw // 2, sh // 2, filter)
    return dst


def mip_chain(l0: np.ndarray, levels: int, filter: int = 0) -> list:
    out = [np.ascontiguousarray(l0)]
    for _ in range(1, levels):
        out.append(mip_level(out[-1], filter))
    return out


def blur(src: np.ndarray, radius: int) -> np.ndarray:
    h, w, ch = src.shape
    dst = np.empty_like(src)
    getattr(lib(), "go_blur_" + _sfx(src.dtype))(_p(src), _p(dst), w, h, ch, radius)
    return dst


def blur_pyramid(levels: list) -> list:
    """SSVGIRenderer.h:209-221: radius 0 at level 0, 2 above."""
    return [blur(l, 0 if k == 0 else 2) for k, l in enumerate(levels)]


def deinterleave_map(w: int, h: int, gx: int = 4, gy: int = 4) -> np.ndarray:
    m = np.empty(w * h, np.int32)
    lib().go_deinterleave_map(w, h, gx, gy, _p(m))
    return m


def interleave_map(w: int, h: int, gx: int = 4, gy: int = 4) -> np.ndarray:
    m = np.empty(w * h, np.int32)
    lib().go_interleave_map(w, h, gx, gy, _p(m))
    return m


def deinterleave(src: np.ndarray, gx: int = 4, gy: int = 4) -> np.ndarray:
    h, w, ch = src.shape
    return src.reshape(h * w, ch)[deinterleave_map(w, h, gx, gy)].reshape(h, w, ch)


def interleave(src: np.ndarray, gx: int = 4, gy: int = 4) -> np.ndarray:
    h, w, ch = src.shape
    return src.reshape(h * w, ch)[interleave_map(w, h, gx, gy)].reshape(h, w, ch)


def _pack(levels: list, dtype) -> np.ndarray:
    return np.ascontiguousarray(np.concatenate([np.asarray(l, dtype).ravel() for l in levels]))


TEX_DEPTH = 1  # march step taps through the texture units' fixed point (sampler.h texture_lod_unit)
TEX_LIGHT = 2


def march(view: GiView, dirs: int, cap: int, light_levels: list, depth_levels: list, normal, ndc, pixels=None,
          pattern: int = 4, dtype=np.float32, step_dirs: int = 0, soft: bool = False, tex: int = 0,
          lod_trace: bool = False):
    """A7 (indirectLighting.frag:114-271).  pixels: optional (n, 2) int array of (x, y);
    step_dirs: direction count of the step and mip formulas (0 = dirs); soft: the
    depth-variance horizon update (SoftHorizon in gi_oracle.cpp); tex: TEX_DEPTH |
    TEX_LIGHT, which step taps go through the texture-unit sampler (fp32 only); lod_trace
    (fp32 only): also return, per pixel, the count, sum and sum of squares of the
    1-based first mip level of the depth taps -- (out, steps, trace)."""
    dtype = np.dtype(dtype)
    L = _pack(light_levels, dtype)
    D = _pack(depth_levels, dtype)
    nrm = np.ascontiguousarray(normal, dtype)
    z = np.ascontiguousarray(ndc, dtype)
    if pixels is None:
        n = view.width * view.height
        pix = None
    else:
        pix = np.ascontiguousarray(pixels, np.int32)
        n = pix.shape[0]
    out = np.zeros((n, 4), dtype)
    steps = np.zeros(n, np.int32)
    trace = np.zeros((n, 3), np.int64) if lod_trace else None
    if dtype == np.float32:
        lib().go_march_f32(C.byref(view), dirs, cap, pattern, _p(L), _p(D), len(light_levels), _p(nrm), _p(z),
                           None if pix is None else _p(pix), C.c_int(n), _p(out), _p(steps), C.c_int(step_dirs),
                           C.c_int(int(soft)), C.c_int(int(tex)), None if trace is None else _p(trace))
    else:
        assert not tex, "the texture-unit sampler is restated in fp32 only"
        lib().go_march_f64(C.byref(view), dirs, cap, pattern, _p(L), _p(D), len(light_levels), _p(nrm), _p(z),
                           None if pix is None else _p(pix), C.c_int(n), _p(out), _p(steps), C.c_int(step_dirs),
                           C.c_int(int(soft)))
    if pixels is None:
        out = out.reshape(view.height, view.width, 4)
    if lod_trace:
        return out, steps, trace
    return out, steps


def _texture_lod(levels: list, coords, lods, out_channels: int, unit: int) -> np.ndarray:
    h, w, ch = np.asarray(levels[0]).shape
    P = _pack(levels, np.float32)
    st = np.ascontiguousarray(coords, np.float32)
    lod = np.ascontiguousarray(lods, np.float32)
    n = lod.shape[0]
    out = np.zeros((n, out_channels), np.float32)
    lib().go_texture_lod_f32(_p(P), w, h, ch, len(levels), _p(st), _p(lod), C.c_int(n), out_channels, _p(out),
                             C.c_int(unit))
    return out


def texture_unit(levels: list, coords, lods, out_channels: int) -> np.ndarray:
    """texture_lod_unit (sampler.h) at n points: the texture units' fixed-point
    trilinear fetch from an fp32 pyramid; coords [n, 2], lods [n]."""
    return _texture_lod(levels, coords, lods, out_channels, 1)


def texture_unit_exact(levels: list, coords, lods, out_channels: int) -> np.ndarray:
    """texture_lod (sampler.h, the Vulkan formulas in fp32) at the same points."""
    return _texture_lod(levels, coords, lods, out_channels, 0)


def march_deinterleaved(view: GiView, dirs: int, cap: int, light_levels, depth_levels, normal_d, ndc_d,
                        pattern: int = 4):
    L = _pack(light_levels, np.float32)
    D = _pack(depth_levels, np.float32)
    out = np.zeros((view.height, view.width, 4), np.float32)
    lib().go_march_deint_f32(C.byref(view), dirs, cap, pattern, _p(L), _p(D), len(light_levels),
                             _p(np.ascontiguousarray(normal_d, np.float32)),
                             _p(np.ascontiguousarray(ndc_d, np.float32)), _p(out))
    return out


def bilateral(indirect, moments, normal) -> np.ndarray:
    h, w, _ = indirect.shape
    out = np.empty((h, w, 4), indirect.dtype)
    getattr(lib(), "go_bilateral_" + _sfx(indirect.dtype))(_p(indirect), _p(moments), _p(normal), _p(out), w, h)
    return out


def denoise(noisy, moments, radius: int) -> np.ndarray:
    h, w, _ = noisy.shape
    out = np.empty((h, w, 4), noisy.dtype)
    getattr(lib(), "go_denoise_" + _sfx(noisy.dtype))(_p(noisy), _p(moments), _p(out), w, h, radius)
    return out


def final_gather(direct, indirect, albedo) -> np.ndarray:
    h, w, _ = direct.shape
    out = np.empty((h, w, 4), direct.dtype)
    getattr(lib(), "go_final_gather_" + _sfx(direct.dtype))(_p(direct), _p(indirect), _p(albedo), _p(out), w, h)
    return out


def gbuffer(view: GiView, prims, dtype=np.float32):
    w, h = view.width, view.height
    a = np.empty((h, w, 4), dtype)
    e = np.empty((h, w, 4), dtype)
    n = np.empty((h, w, 4), dtype)
    m = np.empty((h, w, 2), dtype)
    z = np.empty((h, w, 1), dtype)
    getattr(lib(), "go_gbuffer_" + _sfx(dtype))(C.byref(view), prims, len(prims), _p(a), _p(e), _p(n), _p(m), _p(z))
    return {"albedo": a, "emissive": e, "normal": n, "moments": m, "ndc": z}


def gbuffer_mesh(view: GiView, objects, triangles, prims=None, cull=1, dtype=np.float32):
    """gbuffer over analytic primitives (optional) and a scene's triangle meshes
    (numpy arrays with the gi_mesh_object / gi_triangle layouts)."""
    w, h = view.width, view.height
    a = np.empty((h, w, 4), dtype)
    e = np.empty((h, w, 4), dtype)
    n = np.empty((h, w, 4), dtype)
    m = np.empty((h, w, 2), dtype)
    z = np.empty((h, w, 1), dtype)
    objects = np.ascontiguousarray(objects)
    triangles = np.ascontiguousarray(triangles)
    getattr(lib(), "go_gbuffer_mesh_" + _sfx(dtype))(C.byref(view), prims, 0 if prims is None else len(prims),
                                                     _p(objects), len(objects), _p(triangles), int(cull), _p(a),
                                                     _p(e), _p(n), _p(m), _p(z))
    return {"albedo": a, "emissive": e, "normal": n, "moments": m, "ndc": z}


def shadow_map_mesh(light_view: GiView, objects, triangles, prims=None, cull=1, dtype=np.float32) -> np.ndarray:
    out = np.empty((light_view.height, light_view.width, 1), dtype)
    objects = np.ascontiguousarray(objects)
    triangles = np.ascontiguousarray(triangles)
    getattr(lib(), "go_shadow_mesh_" + _sfx(dtype))(C.byref(light_view), prims, 0 if prims is None else len(prims),
                                                    _p(objects), len(objects), _p(triangles), int(cull), _p(out))
    return out


def shadow_map(light_view: GiView, prims, dtype=np.float32) -> np.ndarray:
    out = np.empty((light_view.height, light_view.width, 1), dtype)
    getattr(lib(), "go_shadow_" + _sfx(dtype))(C.byref(light_view), prims, len(prims), _p(out))
    return out


def direct_light(view: GiView, light_view: GiView, gb: dict, shadow) -> np.ndarray:
    w, h = view.width, view.height
    dtype = gb["albedo"].dtype
    out = np.empty((h, w, 4), dtype)
    getattr(lib(), "go_direct_" + _sfx(dtype))(C.byref(view), C.byref(light_view), _p(gb["albedo"]),
                                               _p(gb["emissive"]), _p(gb["normal"]), _p(gb["ndc"]), _p(shadow),
                                               shadow.shape[0], _p(out))
    return out


def render_frame(view: GiView, gb: dict, direct, dirs: int, cap: int, bounces: int = 1, use_bilateral=True,
                 denoise_radius=0, mip_levels=10, pattern=4, source=None, texture: bool = False,
                 recorded: bool = True):
    """The GI segment of SSVGIRenderer::RenderFrame (SSVGIRenderer.h:207-342), as the CUDA renderer runs it.
    source: the first bounce's light (default: the direct light); temporal feedback passes the
    previous frame's gathered image.  texture: the renderer's GI_MARCH_TEXTURE precision -- the
    depth taps of every bounce through the texture-unit sampler, the light taps of the first
    bounce too; later bounces re-light the first one's recorded march with software light taps
    (recorded=False: a march table of more than 64 steps, every bounce marches with both taps
    through the texture units)."""
    w, h = view.width, view.height
    L = mip_level_count(w, h, mip_levels)
    depth_blur = blur_pyramid(mip_chain(gb["moments"], L))
    src = direct if source is None else source
    out = {}
    for b in range(bounces):
        light_blur = blur_pyramid(mip_chain(src, L))
        tex = 0
        if texture:
            tex = TEX_DEPTH | (TEX_LIGHT if (b == 0 or not recorded) else 0)
        ind, _ = march(view, dirs, cap, light_blur, depth_blur, gb["normal"], gb["ndc"], pattern=pattern,
                       dtype=direct.dtype, tex=tex)
        cur = ind
        if use_bilateral:
            cur = bilateral(cur, gb["moments"], gb["normal"])
        if denoise_radius:
            cur = denoise(cur, gb["moments"], denoise_radius)
        src = final_gather(direct, cur, gb["albedo"])
        out[f"indirect{b}"] = cur
    out["lit"] = src
    return out
