// sampler.h -- Vulkan sampler arithmetic for the CPU oracle (test infrastructure).
//
// Follows the public Vulkan 1.1 specification, chapter "Texel Filtering" and
// "Texel Coordinate Transformation":
//   u = s * width;  i0 = floor(u - 1/2);  alpha = frac(u - 1/2);  i1 = i0 + 1
//   clamp-to-edge:  i = clamp(i, 0, width - 1)
//   linear: tau = (1-a)(1-b) t00 + a(1-b) t10 + (1-a) b t01 + a b t11
//   mipmapMode linear: lambda clamped to [0, q], q = levels - 1;
//     d_lo = floor(lambda), d_hi = min(d_lo + 1, q), delta = frac(lambda);
//     tau = (1 - delta) tau_lo + delta tau_hi; delta == 0 reads d_lo only.
// Hardware filtering uses reduced-precision fixed-point weights; this file uses
// the element type throughout, and the CUDA kernels evaluate the same sequence.
// Weights are summed in the order t00, t10, t01, t11.
// Missing channels of 1- and 2-channel images read as (0, 0, 0, 1), the
// Vulkan rule for converting a format with fewer components to RGBA.
// Compare sampling (sampler2DShadow, compareOp LESS_OR_EQUAL assumed: the
// reference's sampler object is in an absent library) returns the same bilinear
// blend of per-texel pass/fail values.
#pragma once

#include "glsl.h"

namespace oracle {

using namespace glsl;

template <typename T> struct Img {
  const T* p = nullptr;
  int w = 0, h = 0, ch = 0;
  Img() {}
  Img(const T* p_, int w_, int h_, int ch_) : p(p_), w(w_), h(h_), ch(ch_) {}
  vec4<T> fetch(int x, int y) const {
    const T* q = p + ((size_t)y * w + x) * ch;
    vec4<T> r(T(0), T(0), T(0), T(1));
    r.x = q[0];
    if (ch > 1) r.y = q[1];
    if (ch > 2) r.z = q[2];
    if (ch > 3) r.w = q[3];
    return r;
  }
  vec4<T> fetch_clamped(int x, int y) const {
    return fetch(std::min(std::max(x, 0), w - 1), std::min(std::max(y, 0), h - 1));
  }
};

template <typename T> struct Pyr {
  Img<T> lv[16];
  int n = 0;
};

template <typename T> inline void bilinear_setup(T s, int w, int& i0, int& i1, T& a) {
  T u = s * T(w);
  T uu = u - T(0.5);
  T f = std::floor(uu);
  a = uu - f;
  // Clamp before the integer conversion so NaN and huge coordinates map to a
  // defined index (fmin/fmax return the non-NaN operand), as on the device.
  i0 = (int)std::fmin(std::fmax(f, T(-1e6)), T(1e6));
  i1 = i0 + 1;
  i0 = std::min(std::max(i0, 0), w - 1);
  i1 = std::min(std::max(i1, 0), w - 1);
}

template <typename T> inline vec4<T> bilinear(const Img<T>& im, vec2<T> st) {
  int i0, i1, j0, j1;
  T a, b;
  bilinear_setup(st.x, im.w, i0, i1, a);
  bilinear_setup(st.y, im.h, j0, j1, b);
  T oa = T(1) - a, ob = T(1) - b;
  T w00 = oa * ob, w10 = a * ob, w01 = oa * b, w11 = a * b;
  vec4<T> t00 = im.fetch(i0, j0), t10 = im.fetch(i1, j0), t01 = im.fetch(i0, j1), t11 = im.fetch(i1, j1);
  return t00 * w00 + t10 * w10 + t01 * w01 + t11 * w11;
}

// textureLod(sampler2D, st, lod) with linear/linear/clamp-to-edge.
template <typename T> inline vec4<T> texture_lod(const Pyr<T>& py, vec2<T> st, T lod) {
  T q = T(py.n - 1);
  T lam = std::min(std::max(lod, T(0)), q);
  T lo = std::floor(lam);
  T delta = lam - lo;
  int ilo = (int)lo;
  if (delta == T(0)) return bilinear(py.lv[ilo], st);
  int ihi = std::min(ilo + 1, py.n - 1);
  vec4<T> tlo = bilinear(py.lv[ilo], st);
  vec4<T> thi = bilinear(py.lv[ihi], st);
  return tlo * (T(1) - delta) + thi * delta;
}

// Single-level image through a linear sampler at lod 0 (magnification).
template <typename T> inline vec4<T> texture_lod0(const Img<T>& im, vec2<T> st) { return bilinear(im, st); }

// sampler2DShadow, linear filter, compare LESS_OR_EQUAL: lit where ref <= texel.
template <typename T> inline T texture_shadow(const Img<T>& im, vec3<T> c) {
  int i0, i1, j0, j1;
  T a, b;
  bilinear_setup(c.x, im.w, i0, i1, a);
  bilinear_setup(c.y, im.h, j0, j1, b);
  T oa = T(1) - a, ob = T(1) - b;
  T w00 = oa * ob, w10 = a * ob, w01 = oa * b, w11 = a * b;
  T r = c.z;
  T p00 = r <= im.fetch(i0, j0).x ? T(1) : T(0);
  T p10 = r <= im.fetch(i1, j0).x ? T(1) : T(0);
  T p01 = r <= im.fetch(i0, j1).x ? T(1) : T(0);
  T p11 = r <= im.fetch(i1, j1).x ? T(1) : T(0);
  return p00 * w00 + p10 * w10 + p01 * w01 + p11 * w11;
}

}  // namespace oracle
