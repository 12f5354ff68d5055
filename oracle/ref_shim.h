// ref_shim.h -- the GLSL environment in which oracle/_ref compiles the
// reference's own fragment shaders as C++ (test infrastructure).
//
// oracle/build_ref.py reads each shader from the reference checkout, applies a
// short list of mechanical GLSL -> C++ rewrites (listed there) and wraps its
// source in a struct deriving from FragmentShader; this header supplies what the
// shader expects from a Vulkan implementation:
//   * vector and matrix types and built-in functions: the reference's vendored
//     glm (dependencies/glm, 0.9.9), which it already uses on the host to build
//     the very matrices the shaders receive (SSVGIRenderer.h:54-59, Scene.h:30-33);
//     operator swizzles (v.xy, v.rgb) through GLM_FORCE_SWIZZLE;
//   * GLSL's implicit int -> float conversion in the built-ins the shaders call
//     with mixed arguments (max(0, x), smoothstep(0, 1, x));
//   * sampler2D / sampler2DShadow and textureLod / texelFetch / texture: the
//     sampler formulas of oracle/sampler.h (Vulkan specification, linear filter,
//     linear mipmapping, clamp-to-edge; nearest texelFetch), on images the test
//     hands in as fp32 pyramids;
//   * gl_FragCoord (pixel centre) and the screen-quad varying fragScreenCoord
//     ((pixel + 0.5) / viewport, Common/screenspaceQuad.vert:11-19).
// Transcendentals are glm's, i.e. the C++ standard library's (libm): an
// independent evaluation from the project's own fixed-order functions.
#pragma once

#define GLM_FORCE_SWIZZLE
#define GLM_FORCE_RADIANS
#define GLM_FORCE_DEPTH_ZERO_TO_ONE
#define GLM_ENABLE_EXPERIMENTAL
#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>
#include <glm/gtc/type_ptr.hpp>
#include <glm/gtx/transform.hpp>

#include <cstdint>

#include "sampler.h"

namespace refglsl {

using namespace glm;

// GLSL converts int arguments of float built-ins implicitly.
inline float max(int a, float b) { return glm::max((float)a, b); }
inline float max(float a, int b) { return glm::max(a, (float)b); }
inline float max(float a, float b) { return glm::max(a, b); }
inline float min(int a, float b) { return glm::min((float)a, b); }
inline float min(float a, int b) { return glm::min(a, (float)b); }
inline float min(float a, float b) { return glm::min(a, b); }
inline float smoothstep(int a, int b, float x) { return glm::smoothstep((float)a, (float)b, x); }

// Built-ins called with a swizzle (dot(co.xy, v) in indirectLighting.frag's rand):
// glm's templates do not deduce through the swizzle proxy, GLSL takes the vector.
template <int N, typename T, glm::qualifier Q, int E0, int E1, int E2, int E3>
inline T dot(const glm::detail::_swizzle<N, T, Q, E0, E1, E2, E3>& a, const glm::vec<N, T, Q>& b) {
  return glm::dot(glm::vec<N, T, Q>(a), b);
}
template <int N, typename T, glm::qualifier Q, int E0, int E1, int E2, int E3>
inline T length(const glm::detail::_swizzle<N, T, Q, E0, E1, E2, E3>& a) {
  return glm::length(glm::vec<N, T, Q>(a));
}

// GLSL's inverse(mat4): glm's float evaluation (what a shader compiler emits, in
// float), or -- g_inverse_in_double -- the inverse of the same float matrix
// evaluated in double and rounded to float, the way the library and the oracle
// hoist the shader's per-pixel inverses to the host.  Either is a valid GLSL
// inverse(); the tests run the shader both ways to separate the estimator's
// arithmetic from the conditioning of the perspective matrices.
inline bool g_inverse_in_double = false;
inline mat4 inverse(const mat4& m) {
  if (!g_inverse_in_double) return glm::inverse(m);
  glm::dmat4 d;
  for (int c = 0; c < 4; c++)
    for (int r = 0; r < 4; r++) d[c][r] = (double)m[c][r];
  const glm::dmat4 inv = glm::inverse(d);
  mat4 out;
  for (int c = 0; c < 4; c++)
    for (int r = 0; r < 4; r++) out[c][r] = (float)inv[c][r];
  return out;
}

// Per-pixel record of the mip levels a sampler's textureLod calls select:
// count, sum of (level + 1) and sum of (level + 1)^2 (level = floor of the clamped
// LOD, the level the LINEAR mipmap mode reads first).
struct LodTrace {
  long long count = 0, sum = 0, sum2 = 0;
};

struct sampler2D {
  oracle::Pyr<float> pyr;
  LodTrace* trace = nullptr;
};
struct sampler2DShadow {
  oracle::Img<float> img;
};

inline vec4 to_glm(const oracle::vec4<float>& v) { return vec4(v.x, v.y, v.z, v.w); }

inline vec4 textureLod(const sampler2D& s, vec2 st, float lod) {
  if (s.trace) {
    const float q = (float)(s.pyr.n - 1);
    const float lam = std::min(std::max(lod, 0.0f), q);
    const long long lv = (long long)std::floor(lam) + 1;
    s.trace->count += 1;
    s.trace->sum += lv;
    s.trace->sum2 += lv * lv;
  }
  return to_glm(oracle::texture_lod(s.pyr, oracle::vec2<float>(st.x, st.y), lod));
}
inline vec4 textureLod(const sampler2D& s, vec2 st, int lod) { return textureLod(s, st, (float)lod); }
inline vec4 texture(const sampler2D& s, vec2 st) { return textureLod(s, st, 0.0f); }
inline vec4 texelFetch(const sampler2D& s, ivec2 p, int lod) { return to_glm(s.pyr.lv[lod].fetch(p.x, p.y)); }
inline vec4 texture(const sampler2DShadow& s, vec3 c) {
  const float r = oracle::texture_shadow(s.img, oracle::vec3<float>(c.x, c.y, c.z));
  return vec4(r, r, r, r);
}

// gl_FragCoord with .xy as a vector member (the shaders convert it with
// ivec2(gl_FragCoord.xy), which glm's constructors do not take from a swizzle proxy).
struct FragCoord {
  vec2 xy = vec2(0.0f);
  float x = 0.0f, y = 0.0f, z = 0.0f, w = 1.0f;
};

struct FragmentShader {
  FragCoord gl_FragCoord;
};

}  // namespace refglsl
