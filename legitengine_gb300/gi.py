"""ctypes binding of the C ABI in include/legit_gi.h.

Functions take torch CUDA tensors (fp32, contiguous) and pass their device
pointers and the current CUDA stream to the library.  Nothing here computes:
every call is one C-ABI call, and a missing library raises instead of falling
back to another implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import Sequence

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "libgi_gb300.so"

GI_OK = 0
GI_ERR_INVALID_ARGUMENT, GI_ERR_CUDA, GI_ERR_OUT_OF_MEMORY, GI_ERR_UNSUPPORTED, GI_ERR_TIMEOUT, GI_ERR_IO = 1, 2, 3, 4, 5, 6
GI_MAX_LEVELS = 16
GI_MAX_DIRS = 256
GI_MAX_STEPS = 512
GI_MIP_AVG = 0
GI_MIP_DEPTH = 1
GI_PRIM_ROOM, GI_PRIM_BOX, GI_PRIM_SPHERE = 0, 1, 2

F16 = C.c_float * 16


class GiView(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("view", F16), ("proj", F16), ("view_proj", F16),
                ("inv_view", F16), ("inv_proj", F16), ("inv_view_proj", F16)]


class GiCamera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("hor_angle", C.c_float), ("vert_angle", C.c_float), ("fovy", C.c_float),
                ("znear", C.c_float), ("zfar", C.c_float)]


GI_MARCH_EXACT, GI_MARCH_FAST, GI_MARCH_TEXTURE = 0, 1, 2
GI_MLP_LOSS_SQUARED, GI_MLP_LOSS_ABSOLUTE = 0, 1
GI_OCCLUSION_HARD, GI_OCCLUSION_SOFT = 0, 1


class GiMarchParams(C.Structure):
    _fields_ = [("dirs", C.c_int), ("step_cap", C.c_int), ("pattern_size", C.c_int), ("step_dirs", C.c_int),
                ("precision", C.c_int), ("occlusion", C.c_int)]


class GiPrim(C.Structure):
    _fields_ = [("kind", C.c_int32), ("a", C.c_float * 3), ("b", C.c_float * 3), ("albedo", C.c_float * 4),
                ("emissive", C.c_float * 4), ("pad", C.c_float)]


class GiBatchView(C.Structure):
    _fields_ = [("view", GiView), ("march", GiMarchParams), ("albedo", C.c_void_p), ("normal", C.c_void_p),
                ("depth_moments", C.c_void_p), ("ndc_depth", C.c_void_p), ("direct", C.c_void_p),
                ("out_lit", C.c_void_p), ("out_indirect", C.c_void_p)]


class GiFrameParams(C.Structure):
    _fields_ = [("march", GiMarchParams), ("bounces", C.c_int), ("bilateral", C.c_int), ("denoise_radius", C.c_int),
                ("mip_levels", C.c_int), ("feedback", C.c_int)]


class GiFrameInputs(C.Structure):
    _fields_ = [("albedo", C.c_void_p), ("normal", C.c_void_p), ("depth_moments", C.c_void_p),
                ("ndc_depth", C.c_void_p), ("direct", C.c_void_p)]


class GiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None

_P = C.c_void_p
_I = C.c_int
_SIGS = {
    "gi_abi_version": ([], _I),
    "gi_status_string": ([_I], C.c_char_p),
    "gi_last_error": ([], C.c_char_p),
    "gi_launch_count": ([], C.c_uint64),
    "gi_mip_level_count": ([_I, _I, _I], _I),
    "gi_mip_level_size": ([_I, _I, _I, C.POINTER(_I), C.POINTER(_I)], _I),
    "gi_build_mips": ([_P, _I, _I, _I, _I, _I, _P], _I),
    "gi_blur": ([_P, _P, _I, _I, _I, _I, _P], _I),
    "gi_blur_pyramid": ([_P, _P, _I, _I, _I, _I, _P], _I),
    "gi_deinterleave": ([_P, _P, _I, _I, _I, _I, _I, _P], _I),
    "gi_interleave": ([_P, _P, _I, _I, _I, _I, _I, _P], _I),
    "gi_view_from_camera": ([C.POINTER(GiCamera), _I, _I, C.POINTER(GiView)], _I),
    "gi_march": ([C.POINTER(GiView), C.POINTER(GiMarchParams), _P, _P, _I, _P, _P, _P, _P], _I),
    "gi_march_deinterleaved": ([C.POINTER(GiView), C.POINTER(GiMarchParams), _P, _P, _I, _P, _P, _P, _P], _I),
    "gi_bilateral": ([_P, _P, _P, _P, _I, _I, _P], _I),
    "gi_denoise": ([_P, _P, _P, _P, _I, _I, _I, _P], _I),
    "gi_final_gather": ([_P, _P, _P, _P, _I, _I, _P], _I),
    "gi_scene_generate": ([C.c_uint64, _I, _I, C.POINTER(GiPrim), _I, C.POINTER(_I)], _I),
    "gi_scene_light": ([C.POINTER(GiCamera)], _I),
    "gi_camera_spline": ([C.c_uint64, _I, _I, C.POINTER(GiCamera)], _I),
    "gi_camera_spline_in_scene": ([C.c_uint64, C.POINTER(GiPrim), _I, _I, _I, C.POINTER(GiCamera)], _I),
    "gi_gbuffer": ([C.POINTER(GiView), _P, _I, _P, _P, _P, _P, _P, _P], _I),
    "gi_shadow_map": ([C.POINTER(GiView), _P, _I, _P, _P], _I),
    "gi_scene_load": ([C.c_char_p, C.POINTER(_P)], _I),
    "gi_scene_info": ([_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)], _I),
    "gi_scene_copy": ([_P, _P, _P], _I),
    "gi_scene_object_mesh": ([_P, _I], C.c_char_p),
    "gi_scene_destroy": ([_P], _I),
    "gi_gbuffer_mesh": ([C.POINTER(GiView), _P, _I, _P, _I, _P, _I, _I, _P, _P, _P, _P, _P, _P], _I),
    "gi_shadow_map_mesh": ([C.POINTER(GiView), _P, _I, _P, _I, _P, _I, _I, _P, _P], _I),
    "gi_direct_light": ([C.POINTER(GiView), C.POINTER(GiView), _P, _P, _P, _P, _P, _I, _P, _P], _I),
    "gi_march_tile_grid": ([_I, _I, _I, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)], _I),
    "gi_march_tiles": ([C.POINTER(GiView), C.POINTER(GiMarchParams), _P, _P, _I, _P, _P, _P, _P, _I, _P], _I),
    "gi_mlp_param_count": ([], _I),
    "gi_mlp_create": ([C.POINTER(_P)], _I),
    "gi_mlp_destroy": ([_P], _I),
    "gi_mlp_init": ([_P, C.c_uint64], _I),
    "gi_mlp_set_params": ([_P, _P, _I], _I),
    "gi_mlp_get_params": ([_P, _P, _I], _I),
    "gi_mlp_forward": ([_P, _P, _P, _I, _P, _P], _I),
    "gi_mlp_train_step": ([_P, _P, _P, _P, _I, C.c_float, C.POINTER(C.c_float), _P], _I),
    "gi_mlp_set_loss": ([_P, _I], _I),
    "gi_mlp_gradients": ([_P, _P, _P, _P, _I, _P, C.POINTER(C.c_float), _P], _I),
    "gi_mlp_gradients_noalloc": ([_P, _P, _P, _P, _I, _P, _P, _P], _I),
    "gi_mlp_save": ([_P, C.c_char_p], _I),
    "gi_mlp_load": ([_P, C.c_char_p], _I),
    "gi_features": ([_I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I, _P], _I),
    "gi_gather_tiles": ([_P, _I, _I, _I, _P, _I, _P, _P], _I),
    "gi_scatter_tiles": ([_P, _I, _I, _I, _P, _I, _P, _P], _I),
    "gi_march_autotune": ([C.POINTER(GiView), C.POINTER(GiMarchParams), _P, _P, _I, _P, _P, _P, C.POINTER(_I),
                           C.POINTER(_I), C.POINTER(C.c_float), _P], _I),
    "gi_march_tuned_rows": ([_I, _I, _I, _I, _I], _I),
    "gi_march_tuned_layout": ([_I, _I, _I, _I, _I, _I, C.POINTER(_I), C.POINTER(_I)], _I),
    "gi_march_set_layout": ([_I, _I, _I, _I, _I, _I, _I, _I], _I),
    "gi_debug_tensor_core_wait_limit": ([C.c_longlong], _I),
    "gi_debug_fail_allocations": ([_I], _I),
    "gi_debug_live_allocations": ([C.POINTER(C.c_longlong)], _I),
    "gi_texture_sample": ([_P, _I, _I, _I, _I, _I, _P, _P, _I, _P, _P], _I),
    "gi_mlp_reconstruct": ([_P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "gi_mlp_tensor_core_errors": ([C.POINTER(_I)], _I),
    "gi_batch_create": ([C.POINTER(GiBatchView), _I, _I, C.POINTER(_P)], _I),
    "gi_batch_render": ([_P, _P], _I),
    "gi_batch_info": ([_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_float)], _I),
    "gi_batch_destroy": ([_P], _I),
    "gi_batch_set_learned": ([_P, _P, _I, _I, _I, C.c_float], _I),
    "gi_batch_finetune": ([_P, _P, _I, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float), _P], _I),
    "gi_batch_stats": ([_P, C.POINTER(_I), C.POINTER(_I)], _I),
    "gi_renderer_create": ([_I, _I, C.POINTER(GiFrameParams), C.POINTER(_P)], _I),
    "gi_renderer_destroy": ([_P], _I),
    "gi_renderer_set_learned": ([_P, _P, _I, _I, _I, C.c_float], _I),
    "gi_renderer_stats": ([_P, C.POINTER(_I), C.POINTER(_I)], _I),
    "gi_renderer_render": ([_P, C.POINTER(GiView), C.POINTER(GiFrameInputs), _P, _P, _P], _I),
    "gi_renderer_render_host": ([_P, C.POINTER(GiView), _P, _P, _P, _P, _P, _P, _P], _I),
    "gi_renderer_render_host_async": ([_P, C.POINTER(GiView), _P, _P, _P, _P, _P, _P, _P], _I),
    "gi_renderer_host_wait": ([_P], _I),
    "gi_renderer_set_profiling": ([_P, _I], _I),
    "gi_renderer_pass_times": ([_P, _I, C.POINTER(C.c_char_p), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                C.POINTER(_I)], _I),
}


def exported_symbols() -> list[str]:
    return sorted(_SIGS)


def lib():
    """Loads the library (built by legitengine_gb300.build); raises if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise FileNotFoundError(f"{LIB_PATH} is missing: run legitengine_gb300.build.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _check(status: int, what: str):
    if status != GI_OK:
        msg = lib().gi_last_error().decode()
        raise GiError(status, f"{what}: {msg}")


# --------------------------------------------------------------------------
# torch helpers (torch is only plumbing: device memory and streams)

def _torch():
    import torch
    return torch


def _stream():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t) -> C.c_void_p:
    if t is None:
        return C.c_void_p(0)
    torch = _torch()
    assert t.is_cuda and t.dtype == torch.float32 and t.is_contiguous(), "expected a contiguous fp32 CUDA tensor"
    return C.c_void_p(t.data_ptr())


def _dptr(t) -> C.c_void_p:
    """Device pointer of any contiguous CUDA tensor (bf16 features, int32 tile lists)."""
    if t is None:
        return C.c_void_p(0)
    assert t.is_cuda and t.is_contiguous(), "expected a contiguous CUDA tensor"
    return C.c_void_p(t.data_ptr())


def _ptrs(ts: Sequence) -> C.Array:
    arr = (C.c_void_p * len(ts))(*[_ptr(t).value for t in ts])
    return arr


def mip_level_count(w: int, h: int, requested: int = 10) -> int:
    return lib().gi_mip_level_count(w, h, requested)


def mip_level_size(w: int, h: int, level: int) -> tuple[int, int]:
    a, b = C.c_int(), C.c_int()
    _check(lib().gi_mip_level_size(w, h, level, C.byref(a), C.byref(b)), "gi_mip_level_size")
    return a.value, b.value


def alloc_pyramid(w: int, h: int, channels: int, levels: int, device="cuda"):
    torch = _torch()
    out = []
    for k in range(levels):
        lw, lh = w >> k, h >> k
        out.append(torch.empty((lh, lw, channels), dtype=torch.float32, device=device))
    return out


def build_mips(levels: Sequence, channels: int, filter: int = GI_MIP_AVG):
    h, w = levels[0].shape[0], levels[0].shape[1]
    _check(lib().gi_build_mips(_ptrs(levels), w, h, channels, len(levels), filter, _stream()), "gi_build_mips")


def blur(src, dst, radius: int):
    h, w, ch = src.shape
    _check(lib().gi_blur(_ptr(src), _ptr(dst), w, h, ch, radius, _stream()), "gi_blur")


def blur_pyramid(src_levels: Sequence, dst_levels: Sequence):
    h, w, ch = src_levels[0].shape
    _check(lib().gi_blur_pyramid(_ptrs(src_levels), _ptrs(dst_levels), w, h, ch, len(src_levels), _stream()),
           "gi_blur_pyramid")


def deinterleave(src, dst, grid=(4, 4)):
    h, w, ch = src.shape
    _check(lib().gi_deinterleave(_ptr(src), _ptr(dst), w, h, ch, grid[0], grid[1], _stream()), "gi_deinterleave")


def interleave(src, dst, grid=(4, 4)):
    h, w, ch = src.shape
    _check(lib().gi_interleave(_ptr(src), _ptr(dst), w, h, ch, grid[0], grid[1], _stream()), "gi_interleave")


def view_from_camera(cam: GiCamera, w: int, h: int) -> GiView:
    v = GiView()
    _check(lib().gi_view_from_camera(C.byref(cam), w, h, C.byref(v)), "gi_view_from_camera")
    return v


def march(view: GiView, params: GiMarchParams, light_levels, depth_levels, normal, ndc, out, deinterleaved=False):
    fn = lib().gi_march_deinterleaved if deinterleaved else lib().gi_march
    _check(fn(C.byref(view), C.byref(params), _ptrs(light_levels), _ptrs(depth_levels), len(light_levels),
              _ptr(normal), _ptr(ndc), _ptr(out), _stream()), "gi_march")


def bilateral(indirect, depth_moments, normal, out):
    h, w, _ = indirect.shape
    _check(lib().gi_bilateral(_ptr(indirect), _ptr(depth_moments), _ptr(normal), _ptr(out), w, h, _stream()),
           "gi_bilateral")


def denoise(noisy, depth_moments, normal, out, radius: int):
    h, w, _ = noisy.shape
    _check(lib().gi_denoise(_ptr(noisy), _ptr(depth_moments), _ptr(normal), _ptr(out), w, h, radius, _stream()),
           "gi_denoise")


def final_gather(direct, indirect, albedo, out):
    h, w, _ = direct.shape
    _check(lib().gi_final_gather(_ptr(direct), _ptr(indirect), _ptr(albedo), _ptr(out), w, h, _stream()),
           "gi_final_gather")


def scene_generate(seed: int, num_boxes: int, num_spheres: int):
    n = 1 + num_boxes + num_spheres
    arr = (GiPrim * n)()
    cnt = C.c_int()
    _check(lib().gi_scene_generate(seed, num_boxes, num_spheres, arr, n, C.byref(cnt)), "gi_scene_generate")
    return arr


def scene_light() -> GiCamera:
    c = GiCamera()
    _check(lib().gi_scene_light(C.byref(c)), "gi_scene_light")
    return c


def camera_spline(seed: int, frame: int, num_frames: int, prims=None) -> GiCamera:
    """Camera on the seeded spline; with `prims` the control points avoid the scene's objects."""
    c = GiCamera()
    if prims is None:
        _check(lib().gi_camera_spline(seed, frame, num_frames, C.byref(c)), "gi_camera_spline")
    else:
        _check(lib().gi_camera_spline_in_scene(seed, prims, len(prims), frame, num_frames, C.byref(c)),
               "gi_camera_spline_in_scene")
    return c


def prims_to_device(prims):
    """Copies a GiPrim array into a CUDA byte tensor; returns (tensor, count)."""
    torch = _torch()
    raw = bytes(prims)
    t = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
    return t, len(prims)


def gbuffer(view: GiView, prims_dev, num_prims: int, albedo, emissive, normal, moments, ndc):
    _check(lib().gi_gbuffer(C.byref(view), C.c_void_p(prims_dev.data_ptr()), num_prims, _ptr(albedo), _ptr(emissive),
                            _ptr(normal), _ptr(moments), _ptr(ndc), _stream()), "gi_gbuffer")


def shadow_map(light_view: GiView, prims_dev, num_prims: int, out):
    _check(lib().gi_shadow_map(C.byref(light_view), C.c_void_p(prims_dev.data_ptr()), num_prims, _ptr(out),
                               _stream()), "gi_shadow_map")


class MeshDevice:
    """A loaded scene's objects and triangles (scene.Scene) in device memory."""

    def __init__(self, scene):
        import numpy as np
        torch = _torch()
        self.objects = torch.from_numpy(scene.objects.view(np.uint8).copy()).cuda()
        self.triangles = torch.from_numpy(scene.triangles.view(np.uint8).copy()).cuda()
        self.num_objects = len(scene.objects)
        self.num_triangles = len(scene.triangles)

    def _args(self):
        return (C.c_void_p(self.objects.data_ptr()), self.num_objects, C.c_void_p(self.triangles.data_ptr()),
                self.num_triangles)


GI_CULL_NONE, GI_CULL_BACK = 0, 1


def gbuffer_mesh(view: GiView, mesh: MeshDevice, albedo, emissive, normal, moments, ndc, prims_dev=None,
                 num_prims: int = 0, cull: int = GI_CULL_BACK):
    """G-buffer over analytic primitives (optional) and a loaded scene's meshes."""
    pp = C.c_void_p(prims_dev.data_ptr()) if prims_dev is not None else C.c_void_p()
    _check(lib().gi_gbuffer_mesh(C.byref(view), pp, num_prims, *mesh._args(), cull, _ptr(albedo), _ptr(emissive),
                                 _ptr(normal), _ptr(moments), _ptr(ndc), _stream()), "gi_gbuffer_mesh")


def shadow_map_mesh(light_view: GiView, mesh: MeshDevice, out, prims_dev=None, num_prims: int = 0,
                    cull: int = GI_CULL_BACK):
    pp = C.c_void_p(prims_dev.data_ptr()) if prims_dev is not None else C.c_void_p()
    _check(lib().gi_shadow_map_mesh(C.byref(light_view), pp, num_prims, *mesh._args(), cull, _ptr(out), _stream()),
           "gi_shadow_map_mesh")


def direct_light(view: GiView, light_view: GiView, albedo, emissive, normal, ndc, shadow, out):
    _check(lib().gi_direct_light(C.byref(view), C.byref(light_view), _ptr(albedo), _ptr(emissive), _ptr(normal),
                                 _ptr(ndc), _ptr(shadow), shadow.shape[0], _ptr(out), _stream()), "gi_direct_light")


class Renderer:
    """The GI segment of SSVGIRenderer::RenderFrame on resident G-buffer images."""

    def __init__(self, w: int, h: int, dirs=16, step_cap=64, bounces=2, bilateral=True, denoise_radius=0,
                 mip_levels=10, pattern=4, step_dirs=0, precision=GI_MARCH_EXACT, occlusion=GI_OCCLUSION_HARD,
                 feedback=False):
        self.w, self.h = w, h
        p = GiFrameParams()
        p.feedback = int(feedback)
        p.march.dirs, p.march.step_cap, p.march.pattern_size = dirs, step_cap, pattern
        p.march.step_dirs, p.march.precision, p.march.occlusion = step_dirs, precision, occlusion
        p.bounces, p.bilateral, p.denoise_radius, p.mip_levels = bounces, int(bilateral), denoise_radius, mip_levels
        self.params = p
        self._h = C.c_void_p()
        _check(lib().gi_renderer_create(w, h, C.byref(p), C.byref(self._h)), "gi_renderer_create")

    def render(self, view: GiView, albedo, normal, moments, ndc, direct, out_lit, out_indirect=None):
        inp = GiFrameInputs(_ptr(albedo).value, _ptr(normal).value, _ptr(moments).value, _ptr(ndc).value,
                            _ptr(direct).value)
        _check(lib().gi_renderer_render(self._h, C.byref(view), C.byref(inp), _ptr(out_lit), _ptr(out_indirect),
                                        _stream()), "gi_renderer_render")

    def render_host(self, view: GiView, albedo, normal, moments, ndc, direct, out_lit, stream=None):
        """Host (CPU, ideally pinned) tensors in and out; waits for completion."""
        def hp(t):
            return C.c_void_p(t.data_ptr())
        s = stream if stream is not None else _stream()
        _check(lib().gi_renderer_render_host(self._h, C.byref(view), hp(albedo), hp(normal), hp(moments), hp(ndc),
                                             hp(direct), hp(out_lit), s), "gi_renderer_render_host")

    def render_host_async(self, view: GiView, albedo, normal, moments, ndc, direct, out_lit, stream=None):
        """Pipelined host-buffer frame (gi_renderer_render_host_async): returns at once;
        this frame's buffers stay in use until the call two frames later or host_wait()."""
        def hp(t):
            return C.c_void_p(t.data_ptr())
        s = stream if stream is not None else _stream()
        _check(lib().gi_renderer_render_host_async(self._h, C.byref(view), hp(albedo), hp(normal), hp(moments),
                                                   hp(ndc), hp(direct), hp(out_lit), s),
               "gi_renderer_render_host_async")

    def set_profiling(self, on: bool = True):
        """Per-pass GPU timing of every frame (gi_renderer_set_profiling)."""
        _check(lib().gi_renderer_set_profiling(self._h, 1 if on else 0), "gi_renderer_set_profiling")

    def pass_times(self):
        """[(pass name, start ms, end ms)] of the last profiled frame (waits for it)."""
        n = C.c_int()
        _check(lib().gi_renderer_pass_times(self._h, 0, None, None, None, C.byref(n)), "gi_renderer_pass_times")
        k = n.value
        names, a, b = (C.c_char_p * k)(), (C.c_float * k)(), (C.c_float * k)()
        _check(lib().gi_renderer_pass_times(self._h, k, names, a, b, C.byref(n)), "gi_renderer_pass_times")
        return [(names[i].decode(), a[i], b[i]) for i in range(k)]

    def host_wait(self):
        """Waits until every pipelined frame's lit image is on the host."""
        _check(lib().gi_renderer_host_wait(self._h), "gi_renderer_host_wait")

    def set_learned(self, mlp, few_dirs=2, few_step_dirs=0, judge_every=64, threshold=0.25):
        """Learned mode with `mlp` (a gi.Mlp), or the plain method with mlp=None."""
        self._mlp = mlp
        h = mlp.handle if mlp is not None else C.c_void_p()
        _check(lib().gi_renderer_set_learned(self._h, h, few_dirs, few_step_dirs, judge_every, threshold),
               "gi_renderer_set_learned")

    def stats(self):
        a, b = C.c_int(), C.c_int()
        _check(lib().gi_renderer_stats(self._h, C.byref(a), C.byref(b)), "gi_renderer_stats")
        return a.value, b.value

    def close(self):
        if self._h:
            lib().gi_renderer_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------
# Tile-list march and the learned reconstructor

def march_tile_grid(w: int, h: int, pattern: int = 4):
    """(tiles_x, tiles_y, tile_w, tile_h) of the march's CTA tiling."""
    a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    _check(lib().gi_march_tile_grid(w, h, pattern, C.byref(a), C.byref(b), C.byref(c), C.byref(d)),
           "gi_march_tile_grid")
    return a.value, b.value, c.value, d.value


def march_tiles(view: GiView, params: GiMarchParams, light_levels, depth_levels, normal, ndc, out, tiles):
    _check(lib().gi_march_tiles(C.byref(view), C.byref(params), _ptrs(light_levels), _ptrs(depth_levels),
                                len(light_levels), _ptr(normal), _ptr(ndc), _ptr(out), _dptr(tiles),
                                tiles.numel(), _stream()), "gi_march_tiles")


def features(moments, normal, albedo, direct, indirect_levels, filtered, depth_blur_l2, out, scale, tiles=None,
             pattern: int = 4):
    """indirect_levels: the few-ray indirect at mip levels (0, 2, 4); out: bf16 [pixels, 32];
    scale: fp32 [pixels], the exposure scale the light features are divided by."""
    h, w = normal.shape[0], normal.shape[1]
    arr = (C.c_void_p * 3)(*[_ptr(t).value for t in indirect_levels])
    _check(lib().gi_features(w, h, pattern, _ptr(moments), _ptr(normal), _ptr(albedo), _ptr(direct), arr,
                             _ptr(filtered), _ptr(depth_blur_l2), _dptr(out), _ptr(scale), _dptr(tiles),
                             0 if tiles is None else tiles.numel(), _stream()), "gi_features")


def gather_tiles(image, tiles, out, pattern: int = 4):
    h, w = image.shape[0], image.shape[1]
    _check(lib().gi_gather_tiles(_ptr(image), w, h, pattern, _dptr(tiles), tiles.numel(), _ptr(out), _stream()),
           "gi_gather_tiles")


def scatter_tiles(values, tiles, image, pattern: int = 4):
    h, w = image.shape[0], image.shape[1]
    _check(lib().gi_scatter_tiles(_ptr(values), w, h, pattern, _dptr(tiles), tiles.numel(), _ptr(image),
                                  _stream()), "gi_scatter_tiles")


class Mlp:
    """The learned reconstructor's network (C ABI gi_mlp_*)."""

    PARAMS = 10627

    def __init__(self, seed: int | None = 0):
        self._h = C.c_void_p()
        _check(lib().gi_mlp_create(C.byref(self._h)), "gi_mlp_create")
        if seed is not None:
            _check(lib().gi_mlp_init(self._h, seed), "gi_mlp_init")

    def set_params(self, flat):
        import numpy as np
        a = np.ascontiguousarray(flat, np.float32)
        _check(lib().gi_mlp_set_params(self._h, a.ctypes.data_as(C.c_void_p), a.size), "gi_mlp_set_params")

    def get_params(self):
        import numpy as np
        a = np.empty(self.PARAMS, np.float32)
        _check(lib().gi_mlp_get_params(self._h, a.ctypes.data_as(C.c_void_p), a.size), "gi_mlp_get_params")
        return a

    def forward(self, feats, out, scale=None):
        _check(lib().gi_mlp_forward(self._h, _dptr(feats), _ptr(scale), feats.shape[0], _ptr(out), _stream()),
               "gi_mlp_forward")

    def set_loss(self, loss: int):
        """GI_MLP_LOSS_SQUARED (default) or GI_MLP_LOSS_ABSOLUTE for train_step and gradients."""
        _check(lib().gi_mlp_set_loss(self._h, loss), "gi_mlp_set_loss")

    def train_step(self, feats, targets, lr=1e-3, want_loss=True, scale=None):
        l = C.c_float()
        _check(lib().gi_mlp_train_step(self._h, _dptr(feats), _ptr(targets), _ptr(scale), feats.shape[0], lr,
                                       C.byref(l) if want_loss else None, _stream()), "gi_mlp_train_step")
        return l.value if want_loss else None

    def gradients(self, feats, targets, scale=None):
        import numpy as np
        g = np.empty(self.PARAMS, np.float32)
        l = C.c_float()
        _check(lib().gi_mlp_gradients(self._h, _dptr(feats), _ptr(targets), _ptr(scale), feats.shape[0],
                                      g.ctypes.data_as(C.c_void_p), C.byref(l), _stream()), "gi_mlp_gradients")
        return l.value, g

    def reconstruct(self, moments, normal, albedo, direct, indirect_levels, filtered, depth_blur_l2, out,
                    pattern: int = 4):
        """Fused features + network on the tcgen05 tensor cores for a whole frame
        (the result of features() followed by forward(), without the feature buffer)."""
        h, w, _ = moments.shape
        _check(lib().gi_mlp_reconstruct(self._h, w, h, pattern, _ptr(moments), _ptr(normal), _ptr(albedo),
                                        _ptr(direct), _ptrs(indirect_levels), _ptr(filtered), _ptr(depth_blur_l2),
                                        _ptr(out), _stream()), "gi_mlp_reconstruct")

    def save(self, path: str):
        _check(lib().gi_mlp_save(self._h, str(path).encode()), "gi_mlp_save")

    def load(self, path: str):
        _check(lib().gi_mlp_load(self._h, str(path).encode()), "gi_mlp_load")

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().gi_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tensor_core_errors() -> int:
    n = C.c_int()
    _check(lib().gi_mlp_tensor_core_errors(C.byref(n)), "gi_mlp_tensor_core_errors")
    return n.value


def march_autotune(view: GiView, params: GiMarchParams, light_levels, depth_levels, normal, ndc, out):
    """Times each launch layout on these inputs and records the fastest; returns
    (rows, rays_per_warp, ms)."""
    r, rpw, ms = C.c_int(), C.c_int(), C.c_float()
    _check(lib().gi_march_autotune(C.byref(view), C.byref(params), _ptrs(light_levels), _ptrs(depth_levels),
                                   len(light_levels), _ptr(normal), _ptr(ndc), _ptr(out), C.byref(r), C.byref(rpw),
                                   C.byref(ms), _stream()), "gi_march_autotune")
    return r.value, rpw.value, ms.value


def march_tuned_layout(width: int, height: int, dirs: int, step_dirs: int, step_cap: int, precision: int):
    """The recorded (rows, rays_per_warp) of a march shape, (0, 0) if never tuned."""
    r, rpw = C.c_int(), C.c_int()
    _check(lib().gi_march_tuned_layout(width, height, dirs, step_dirs, step_cap, precision, C.byref(r),
                                       C.byref(rpw)), "gi_march_tuned_layout")
    return r.value, rpw.value


def march_set_layout(width: int, height: int, dirs: int, step_dirs: int, step_cap: int, precision: int, rows: int,
                     rays_per_warp: int):
    """Records a launch layout for a march shape without timing."""
    _check(lib().gi_march_set_layout(width, height, dirs, step_dirs, step_cap, precision, rows, rays_per_warp),
           "gi_march_set_layout")


def texture_sample(levels, channels: int, coords, lods, out):
    """gi_texture_sample: trilinear fetches through the texture units from a pyramid
    (levels: device tensors [h_k, w_k, c]); coords [n, 2], lods [n], out [n, channels]."""
    h, w, src = levels[0].shape
    _check(lib().gi_texture_sample(_ptrs(levels), w, h, len(levels), channels, src, _ptr(coords), _ptr(lods),
                                   int(lods.shape[0]), _ptr(out), _stream()), "gi_texture_sample")


class Batch:
    """Many views per frame, marched in one persistent launch (C ABI gi_batch_*)."""

    def __init__(self, views, tile_rows: int = 0):
        """views: list of dicts with view (GiView), march (GiMarchParams) and the device tensors
        albedo, normal, moments, ndc, direct, out_lit and optionally out_indirect."""
        arr = (GiBatchView * len(views))()
        self._keep = views
        for i, v in enumerate(views):
            arr[i].view = v["view"]
            arr[i].march = v["march"]
            arr[i].albedo, arr[i].normal = _ptr(v["albedo"]).value, _ptr(v["normal"]).value
            arr[i].depth_moments, arr[i].ndc_depth = _ptr(v["moments"]).value, _ptr(v["ndc"]).value
            arr[i].direct, arr[i].out_lit = _ptr(v["direct"]).value, _ptr(v["out_lit"]).value
            arr[i].out_indirect = _ptr(v.get("out_indirect")).value
        self._h = C.c_void_p()
        _check(lib().gi_batch_create(arr, len(views), tile_rows, C.byref(self._h)), "gi_batch_create")

    def render(self, stream=None):
        _check(lib().gi_batch_render(self._h, stream if stream is not None else _stream()), "gi_batch_render")

    def info(self):
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_float()
        _check(lib().gi_batch_info(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)), "gi_batch_info")
        return {"work_items": a.value, "grid": b.value, "tile_rows": c.value, "tuned_ms": d.value}

    def set_learned(self, mlp, few_dirs=2, few_step_dirs=0, judge_every=64, threshold=0.25):
        """Learned mode with `mlp` (a gi.Mlp, kept alive here), or the plain method with mlp=None."""
        self._mlp = mlp
        h = mlp.handle if mlp is not None else C.c_void_p()
        _check(lib().gi_batch_set_learned(self._h, h, few_dirs, few_step_dirs, judge_every, threshold),
               "gi_batch_set_learned")

    def finetune(self, mlp, target_dirs=256, lr=1e-4, stream=None):
        """One Adam step on the last frame's judged tiles; returns (loss, sampled error)."""
        loss, err = C.c_float(), C.c_float()
        _check(lib().gi_batch_finetune(self._h, mlp.handle, target_dirs, lr, C.byref(loss), C.byref(err),
                                       stream if stream is not None else _stream()), "gi_batch_finetune")
        return loss.value, err.value

    def stats(self):
        a, b = C.c_int(), C.c_int()
        _check(lib().gi_batch_stats(self._h, C.byref(a), C.byref(b)), "gi_batch_stats")
        return a.value, b.value

    def close(self):
        if self._h:
            lib().gi_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def debug_fail_allocations(after: int):
    """Test hook: the next `after` device allocations of the library succeed, later ones fail (-1: off)."""
    _check(lib().gi_debug_fail_allocations(after), "gi_debug_fail_allocations")


def debug_live_allocations() -> int:
    n = C.c_longlong()
    _check(lib().gi_debug_live_allocations(C.byref(n)), "gi_debug_live_allocations")
    return n.value


def debug_tensor_core_wait_limit(cycles: int):
    """Test hook: bound of each tile group's first tensor-core wait in gi_mlp_reconstruct (<= 0: default)."""
    _check(lib().gi_debug_tensor_core_wait_limit(cycles), "gi_debug_tensor_core_wait_limit")
