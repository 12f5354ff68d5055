// glsl.h -- GLSL 4.50 value types and built-ins for the CPU oracle (test
// infrastructure only; the shipped library never includes this file).
//
// Rounding contract shared with the CUDA kernels: every GLSL operator is one
// IEEE-754 operation in the element type, evaluated left to right with no
// contraction (this file is compiled with -ffp-contract=off):
//   dot(a, b)      = ((a.x*b.x + a.y*b.y) + a.z*b.z) [+ a.w*b.w]
//   m * v          = (m[0]*v.x + m[1]*v.y) + (m[2]*v.z + m[3]*v.w)   (columns;
//                    glm's order, which the reference's own shader compiled with
//                    glm follows bit for bit -- oracle/_ref)
//   normalize(v)   = v * (1 / sqrt(dot(v, v)))    (glm's normalize)
//   a / b          = a * RN(1 / b) in fp32 (gdiv); exact division in double
//   cross(a, b)    = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
// Transcendentals come from Math<T>: for float the project's fixed-order
// functions (legitengine_gb300/csrc/gi_math.h), for double the C library.
#pragma once

#include <cmath>
#include <cstdint>
#include <algorithm>

#include "../legitengine_gb300/csrc/gi_math.h"

namespace glsl {

template <typename T> struct Math;

// fp32: the library's fixed-order functions (gi_math.h), the evaluation contract
// the CUDA kernels share.  `libm` switches to the C library's float functions
// and true division -- how the reference's shader evaluates when compiled as C++
// (oracle/_ref) -- so that a test can separate the restatement of the shader from
// the accuracy of the contract's functions; it is off except inside such a test.
template <> struct Math<float> {
  static inline bool libm = false;
  static float log(float x) { return libm ? std::log(x) : gi::logf_(x); }
  static float log2(float x) { return libm ? std::log2(x) : gi::log2f_(x); }
  static float exp(float x) { return libm ? std::exp(x) : gi::expf_(x); }
  static float pow(float b, float e) { return libm ? std::pow(b, e) : gi::powf_(b, e); }
  static float atan2(float y, float x) { return libm ? std::atan2(y, x) : gi::atan2f_(y, x); }
  static float sin(float x) { return libm ? std::sin(x) : gi::sinf_(x); }
  static float cos(float x) { return libm ? std::cos(x) : gi::cosf_(x); }
  static float sqrt(float x) { return std::sqrt(x); }
  static float div(float a, float b) { return libm ? a / b : gi::div_(a, b); }
};

template <> struct Math<double> {
  static double log(double x) { return std::log(x); }
  static double log2(double x) { return std::log2(x); }
  static double exp(double x) { return std::exp(x); }
  static double pow(double b, double e) { return std::pow(b, e); }
  static double atan2(double y, double x) { return std::atan2(y, x); }
  static double sin(double x) { return std::sin(x); }
  static double cos(double x) { return std::cos(x); }
  static double sqrt(double x) { return std::sqrt(x); }
  static double div(double a, double b) { return a / b; }
};

// GLSL division: fp32 is a times the correctly rounded reciprocal of b (the
// library's contract, gi_math.h div_); double divides exactly.
template <typename T> T gdiv(T a, T b) { return Math<T>::div(a, b); }

template <typename T> struct vec2 {
  T x, y;
  vec2() : x(0), y(0) {}
  vec2(T a, T b) : x(a), y(b) {}
  explicit vec2(T a) : x(a), y(a) {}
};
template <typename T> struct vec3 {
  T x, y, z;
  vec3() : x(0), y(0), z(0) {}
  vec3(T a, T b, T c) : x(a), y(b), z(c) {}
  explicit vec3(T a) : x(a), y(a), z(a) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <typename T> struct vec4 {
  T x, y, z, w;
  vec4() : x(0), y(0), z(0), w(0) {}
  vec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
  vec4(vec3<T> v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec4(vec2<T> v, T c, T d) : x(v.x), y(v.y), z(c), w(d) {}
  explicit vec4(T a) : x(a), y(a), z(a), w(a) {}
  vec3<T> xyz() const { return vec3<T>(x, y, z); }
  vec3<T> rgb() const { return vec3<T>(x, y, z); }
  vec2<T> xy() const { return vec2<T>(x, y); }
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

// Column-major 4x4 matrix: c[j] is column j, as in GLSL and glm.
template <typename T> struct mat4 {
  vec4<T> c[4];
  mat4() {}
  static mat4 from_colmajor(const T* m) {
    mat4 r;
    for (int j = 0; j < 4; j++) r.c[j] = vec4<T>(m[4 * j + 0], m[4 * j + 1], m[4 * j + 2], m[4 * j + 3]);
    return r;
  }
};

template <typename T> vec2<T> operator+(vec2<T> a, vec2<T> b) { return vec2<T>(a.x + b.x, a.y + b.y); }
template <typename T> vec2<T> operator-(vec2<T> a, vec2<T> b) { return vec2<T>(a.x - b.x, a.y - b.y); }
template <typename T> vec2<T> operator*(vec2<T> a, vec2<T> b) { return vec2<T>(a.x * b.x, a.y * b.y); }
template <typename T> vec2<T> operator/(vec2<T> a, vec2<T> b) { return vec2<T>(gdiv(a.x, b.x), gdiv(a.y, b.y)); }
template <typename T> vec2<T> operator*(vec2<T> a, T b) { return vec2<T>(a.x * b, a.y * b); }
template <typename T> vec2<T> operator/(vec2<T> a, T b) { return vec2<T>(gdiv(a.x, b), gdiv(a.y, b)); }
template <typename T> vec2<T> operator+(vec2<T> a, T b) { return vec2<T>(a.x + b, a.y + b); }
template <typename T> vec2<T> operator-(vec2<T> a, T b) { return vec2<T>(a.x - b, a.y - b); }

template <typename T> vec3<T> operator+(vec3<T> a, vec3<T> b) { return vec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> vec3<T> operator-(vec3<T> a, vec3<T> b) { return vec3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> vec3<T> operator*(vec3<T> a, vec3<T> b) { return vec3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename T> vec3<T> operator/(vec3<T> a, vec3<T> b) { return vec3<T>(gdiv(a.x, b.x), gdiv(a.y, b.y), gdiv(a.z, b.z)); }
template <typename T> vec3<T> operator*(vec3<T> a, T b) { return vec3<T>(a.x * b, a.y * b, a.z * b); }
template <typename T> vec3<T> operator*(T a, vec3<T> b) { return vec3<T>(a * b.x, a * b.y, a * b.z); }
template <typename T> vec3<T> operator/(vec3<T> a, T b) { return vec3<T>(gdiv(a.x, b), gdiv(a.y, b), gdiv(a.z, b)); }
template <typename T> vec3<T> operator-(vec3<T> a) { return vec3<T>(-a.x, -a.y, -a.z); }

template <typename T> vec4<T> operator+(vec4<T> a, vec4<T> b) { return vec4<T>(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
template <typename T> vec4<T> operator-(vec4<T> a, vec4<T> b) { return vec4<T>(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
template <typename T> vec4<T> operator*(vec4<T> a, vec4<T> b) { return vec4<T>(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
template <typename T> vec4<T> operator*(vec4<T> a, T b) { return vec4<T>(a.x * b, a.y * b, a.z * b, a.w * b); }
template <typename T> vec4<T> operator/(vec4<T> a, T b) { return vec4<T>(gdiv(a.x, b), gdiv(a.y, b), gdiv(a.z, b), gdiv(a.w, b)); }

template <typename T> T dot(vec2<T> a, vec2<T> b) { return a.x * b.x + a.y * b.y; }
template <typename T> T dot(vec3<T> a, vec3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> T dot(vec4<T> a, vec4<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <typename T> vec3<T> cross(vec3<T> a, vec3<T> b) {
  return vec3<T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <typename T> T length(vec3<T> v) { return Math<T>::sqrt(dot(v, v)); }
template <typename T> T length(vec2<T> v) { return Math<T>::sqrt(dot(v, v)); }
template <typename T> vec3<T> normalize(vec3<T> v) {
  const T r = gdiv(T(1), Math<T>::sqrt(dot(v, v)));
  return vec3<T>(v.x * r, v.y * r, v.z * r);
}

template <typename T> vec4<T> operator*(const mat4<T>& m, vec4<T> v) {
  vec4<T> r;
  for (int i = 0; i < 4; i++) r[i] = (m.c[0][i] * v.x + m.c[1][i] * v.y) + (m.c[2][i] * v.z + m.c[3][i] * v.w);
  return r;
}

template <typename T> T clamp(T v, T lo, T hi) { return std::min(std::max(v, lo), hi); }
template <typename T> T saturate(T v) { return clamp(v, T(0), T(1)); }
template <typename T> T fract(T v) { return v - std::floor(v); }
template <typename T> T smoothstep(T e0, T e1, T x) {
  T t = clamp(gdiv(x - e0, e1 - e0), T(0), T(1));
  return t * t * (T(3) - T(2) * t);
}
template <typename T> T mix(T a, T b, T t) { return a * (T(1) - t) + b * t; }

}  // namespace glsl
