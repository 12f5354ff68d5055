"""ctypes binding of oracle/_ref/libgi_ref.so: the reference's own GLSL passes
compiled as C++ by oracle/build_ref.py (test infrastructure).

Only the tests load it, to check the oracle's restatement against the
reference's source.  It exists only where the reference checkout does (the
recipe reads the shaders and glm from there); `available()` says whether it
could be built.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_ref

_lib = None


def available() -> bool:
    return build_ref.available()


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build()
        if path is None:
            raise FileNotFoundError("oracle/_ref needs the reference checkout (see oracle/build_ref.py)")
        _lib = C.CDLL(str(path))
    return _lib


def _p(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _pack(levels):
    return np.ascontiguousarray(np.concatenate([_f32(l).ravel() for l in levels]))


def set_inverse_in_double(on: bool):
    """The shaders' inverse(mat4) in double rounded to float (True) or glm's float (False)."""
    lib().ref_set_inverse_in_double(C.c_int(int(on)))


def mip_level(src, filter: int = 0):
    """Common/mipLevelBuilder.frag over one level: src [h, w, ch] -> [h/2, w/2, ch]."""
    src = _f32(src)
    h, w, ch = src.shape
    dst = np.zeros((max(h // 2, 1), max(w // 2, 1), ch), np.float32)
    lib().ref_mip_level(_p(src), w, h, ch, _p(dst), dst.shape[1], dst.shape[0], C.c_int(filter))
    return dst


def blur(src, radius: int):
    """Common/blurLayerBuilder.frag."""
    src = _f32(src)
    h, w, ch = src.shape
    dst = np.zeros_like(src)
    lib().ref_blur(_p(src), _p(dst), w, h, ch, C.c_int(radius))
    return dst


def permute(src, inverse: bool, gx: int = 4, gy: int = 4):
    """Common/deinterleave.frag (inverse False) or Common/interleave.frag."""
    src = _f32(src)
    h, w, ch = src.shape
    dst = np.zeros_like(src)
    lib().ref_permute(_p(src), _p(dst), w, h, ch, gx, gy, C.c_int(int(inverse)))
    return dst


def indirect(view16, proj16, w: int, h: int, light_levels, depth_levels, normal, ndc, dirs: int = 0, pixels=None):
    """SSVGI/indirectLighting.frag (dirs 0: as written, dirsCount = 4).  Returns
    (rgba [n, 4] or [h, w, 4], trace [n, 3]: count / sum / sum of squares of the
    1-based first mip level of the depth-moment taps)."""
    L, D = _pack(light_levels), _pack(depth_levels)
    nrm, z = _f32(normal), _f32(ndc)
    v, pr = _f32(view16), _f32(proj16)
    if pixels is None:
        n, pix = w * h, None
    else:
        pix = np.ascontiguousarray(pixels, np.int32)
        n = pix.shape[0]
    out = np.zeros((n, 4), np.float32)
    trace = np.zeros((n, 3), np.int64)
    lib().ref_indirect(_p(v), _p(pr), w, h, C.c_int(dirs), _p(L), _p(D), len(light_levels), _p(nrm), _p(z),
                       None if pix is None else _p(pix), C.c_int(n), _p(out), _p(trace))
    if pixels is None:
        out = out.reshape(h, w, 4)
    return out, trace


def final_gather(direct, blurred_levels, albedo, indirect_light):
    """Common/finalGatherer.frag."""
    d, a, i = _f32(direct), _f32(albedo), _f32(indirect_light)
    h, w, _ = d.shape
    B = _pack(blurred_levels)
    out = np.zeros((h, w, 4), np.float32)
    lib().ref_final_gather(_p(d), _p(B), len(blurred_levels), _p(a), _p(i), w, h, _p(out))
    return out


def direct(view16, proj16, light_view16, light_proj16, albedo, emissive, normal, ndc, shadow):
    """Common/directLighting.frag."""
    arrs = [_f32(x) for x in (view16, proj16, light_view16, light_proj16, albedo, emissive, normal, ndc, shadow)]
    h, w, _ = arrs[4].shape
    sh, sw = arrs[8].shape[:2]
    out = np.zeros((h, w, 4), np.float32)
    lib().ref_direct(*[_p(x) for x in arrs], sw, sh, w, h, _p(out))
    return out


def denoise(view16, proj16, noisy, moments, normal, radius: int):
    """Common/denoiser.frag."""
    arrs = [_f32(x) for x in (view16, proj16, noisy, moments, normal)]
    h, w, _ = arrs[2].shape
    out = np.zeros((h, w, 4), np.float32)
    lib().ref_denoise(*[_p(x) for x in arrs], w, h, C.c_int(radius), _p(out))
    return out


def camera_matrices(pos, hor_angle: float, vert_angle: float, fovy: float, aspect: float, znear: float,
                    zfar: float):
    """(view, proj) as float[16] column-major, built with glm as SSVGIRenderer.h:54-59 does."""
    p = _f32(pos)
    view = np.zeros(16, np.float32)
    proj = np.zeros(16, np.float32)
    lib().ref_camera_matrices(_p(p), C.c_float(hor_angle), C.c_float(vert_angle), C.c_float(fovy),
                              C.c_float(aspect), C.c_float(znear), C.c_float(zfar), _p(view), _p(proj))
    return view, proj


def shader_inverses(view16, proj16):
    """(inverse(proj * view), inverse(view)) as the indirect pass's shader computes
    them from its uniforms, float[16] column-major."""
    v, p = _f32(view16), _f32(proj16)
    ivp = np.zeros(16, np.float32)
    iv = np.zeros(16, np.float32)
    lib().ref_shader_inverses(_p(v), _p(p), _p(ivp), _p(iv))
    return ivp, iv
