// gi_device.cuh -- device-side vector arithmetic and Vulkan sampler arithmetic.
//
// Evaluation contract (shared with the host restatement used for testing): each
// GLSL operator is one IEEE-754 fp32 operation, evaluated left to right; no
// multiply-add contraction (the library is compiled with --fmad=false, and the
// only fused operations are the explicit fmaf calls inside gi_math.h);
// square roots are correctly rounded (no fast-math); every division a / b is
// a * rcp_(b) with rcp_ the correctly rounded reciprocal (gi_math.h div_).
//   dot(a, b)    = (a.x*b.x + a.y*b.y) + a.z*b.z
//   M * v        = (c0*v.x + c1*v.y) + (c2*v.z + c3*v.w)     (columns c0..c3;
//                  glm's order: the depth and translation terms of an
//                  unprojection, which nearly cancel, are summed first)
//   normalize(v) = v * (1 / sqrt(dot(v, v)))
// Sampler arithmetic follows the Vulkan specification (Texel Filtering):
//   u = s * w; i0 = floor(u - 0.5); a = frac(u - 0.5); clamp-to-edge;
//   bilinear sum in the order t00, t10, t01, t11; trilinear
//   tlo * (1 - delta) + thi * delta, delta == 0 reading one level.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gi_math.h"

namespace gi {
namespace dev {

struct f2 { float x, y; };
struct f3 { float x, y, z; };

__device__ __forceinline__ f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 mul3s(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 div3s(f3 a, float s) {
  const float r = rcp_(s);
  return mk3(a.x * r, a.y * r, a.z * r);
}
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return mk3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ f3 normalize3(f3 v) {
  const float r = rcp_(sqrtf(dot3(v, v)));
  return mk3(v.x * r, v.y * r, v.z * r);
}
__device__ __forceinline__ float gmin(float a, float b) { return b < a ? b : a; }  // GLSL min
__device__ __forceinline__ float gmax(float a, float b) { return a < b ? b : a; }  // GLSL max
__device__ __forceinline__ float saturate(float v) { return gmin(gmax(v, 0.0f), 1.0f); }
__device__ __forceinline__ int iclamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Column-major 4x4 matrix as stored by glm.
struct Mat4 {
  float m[16];
};

// M * (x, y, z, w); element (row r, column c) is m[4c + r].
__device__ __forceinline__ float4 mat_vec(const Mat4& M, float x, float y, float z, float w) {
  float4 r;
  r.x = (M.m[0] * x + M.m[4] * y) + (M.m[8] * z + M.m[12] * w);
  r.y = (M.m[1] * x + M.m[5] * y) + (M.m[9] * z + M.m[13] * w);
  r.z = (M.m[2] * x + M.m[6] * y) + (M.m[10] * z + M.m[14] * w);
  r.w = (M.m[3] * x + M.m[7] * y) + (M.m[11] * z + M.m[15] * w);
  return r;
}

// Unproject (indirectLighting.frag:20-25).
__device__ __forceinline__ f3 unproject(const Mat4& inv, float sx, float sy, float sz) {
  float4 v = mat_vec(inv, sx * 2.0f - 1.0f, sy * 2.0f - 1.0f, sz, 1.0f);
  const float r = rcp_(v.w);
  return mk3(v.x * r, v.y * r, v.z * r);
}

// Project (indirectLighting.frag:27-34).
__device__ __forceinline__ f3 project(const Mat4& M, f3 p) {
  float4 n = mat_vec(M, p.x, p.y, p.z, 1.0f);
  const float r = rcp_(n.w);
  float x = n.x * r, y = n.y * r, z = n.z * r;
  return mk3(x * 0.5f + 0.5f, y * 0.5f + 0.5f, z);
}

// ---- Fast evaluation (march precision GI_MARCH_FAST) ----------------------
// Explicit fused multiply-adds, the hardware reciprocal square root and
// reciprocal, and a fitted atan, used only inside the fast march's step loop;
// everything that selects an integer (step counts, mip levels, texel indices)
// stays in the exact contract.
__device__ __forceinline__ float fdot3(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
__device__ __forceinline__ f3 fnormalize3(f3 v) {
  const float r = rsqrtf(fdot3(v, v));
  return mk3(v.x * r, v.y * r, v.z * r);
}
__device__ __forceinline__ float4 fmat_vec(const Mat4& M, float x, float y, float z, float w) {
  float4 r;
  r.x = fmaf(M.m[4], y, M.m[0] * x) + fmaf(M.m[8], z, M.m[12] * w);
  r.y = fmaf(M.m[5], y, M.m[1] * x) + fmaf(M.m[9], z, M.m[13] * w);
  r.z = fmaf(M.m[6], y, M.m[2] * x) + fmaf(M.m[10], z, M.m[14] * w);
  r.w = fmaf(M.m[7], y, M.m[3] * x) + fmaf(M.m[11], z, M.m[15] * w);
  return r;
}
__device__ __forceinline__ f3 funproject(const Mat4& inv, float sx, float sy, float sz) {
  const float4 v = fmat_vec(inv, fmaf(sx, 2.0f, -1.0f), fmaf(sy, 2.0f, -1.0f), sz, 1.0f);
  const float r = __fdividef(1.0f, v.w);
  return mk3(v.x * r, v.y * r, v.z * r);
}
// atan2 by octant reduction to t = min(|x|,|y|) / max(|x|,|y|) in [0, 1] and
// atan(t) = t P(t^2), P of degree 8 fitted to atan(t)/t by iteratively reweighted
// least squares on 6000 Chebyshev nodes of [0, 1] (max error 9.4e-8 rad in fp32,
// about one ulp of the result; the quotient's approximate division adds ~2 ulp).
__device__ __forceinline__ float fast_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  const float t = mx > 0.0f ? __fdividef(mn, mx) : 0.0f;
  const float z = t * t;
  float p = 0.0024567246437072754f;
  p = fmaf(p, z, -0.014401359483599663f);
  p = fmaf(p, z, 0.039781227707862854f);
  p = fmaf(p, z, -0.07234857976436615f);
  p = fmaf(p, z, 0.10498946905136108f);
  p = fmaf(p, z, -0.14161229133605957f);
  p = fmaf(p, z, 0.19985906779766083f);
  p = fmaf(p, z, -0.33332598209381104f);
  p = fmaf(p, z, 0.9999998807907104f);
  float r = p * t;
  if (ay > ax) r = 1.5707963267948966f - r;
  if (x < 0.0f) r = 3.1415926535897932f - r;
  return copysignf(r, y);
}

// Linear-filter coordinate setup for one axis; fw == (float)w.
__device__ __forceinline__ void lin_setup_f(float s, float fw, int w, int& i0, int& i1, float& a) {
  float u = s * fw;
  float uu = u - 0.5f;
  float f = floorf(uu);
  a = uu - f;
  int i = (int)fminf(fmaxf(f, -1.0e6f), 1.0e6f);  // NaN and huge coordinates -> defined index
  i0 = iclamp(i, 0, w - 1);
  i1 = iclamp(i + 1, 0, w - 1);
}

__device__ __forceinline__ void lin_setup(float s, int w, int& i0, int& i1, float& a) {
  lin_setup_f(s, (float)w, w, i0, i1, a);
}

struct Bilin {
  int o00, o10, o01, o11;  // texel indices (y * w + x)
  float w00, w10, w01, w11;
};

// Bilinear footprint; fw, fh == (float)w, (float)h.
__device__ __forceinline__ Bilin bilin_f(float s, float t, float fw, float fh, int w, int h) {
  int i0, i1, j0, j1;
  float a, b;
  lin_setup_f(s, fw, w, i0, i1, a);
  lin_setup_f(t, fh, h, j0, j1, b);
  float oa = 1.0f - a, ob = 1.0f - b;
  Bilin r;
  r.w00 = oa * ob;
  r.w10 = a * ob;
  r.w01 = oa * b;
  r.w11 = a * b;
  r.o00 = j0 * w + i0;
  r.o10 = j0 * w + i1;
  r.o01 = j1 * w + i0;
  r.o11 = j1 * w + i1;
  return r;
}

__device__ __forceinline__ Bilin bilin(float s, float t, int w, int h) {
  return bilin_f(s, t, (float)w, (float)h, w, h);
}

__device__ __forceinline__ float blend1(const Bilin& B, float t00, float t10, float t01, float t11) {
  return t00 * B.w00 + t10 * B.w10 + t01 * B.w01 + t11 * B.w11;
}

__device__ __forceinline__ float4 blend4(const Bilin& B, float4 a, float4 b, float4 c, float4 d) {
  float4 r;
  r.x = a.x * B.w00 + b.x * B.w10 + c.x * B.w01 + d.x * B.w11;
  r.y = a.y * B.w00 + b.y * B.w10 + c.y * B.w01 + d.y * B.w11;
  r.z = a.z * B.w00 + b.z * B.w10 + c.z * B.w01 + d.z * B.w11;
  r.w = a.w * B.w00 + b.w * B.w10 + c.w * B.w01 + d.w * B.w11;
  return r;
}

__device__ __forceinline__ float4 ld4(const float* p, int i) { return __ldg(reinterpret_cast<const float4*>(p) + i); }
__device__ __forceinline__ float2 ld2(const float* p, int i) { return __ldg(reinterpret_cast<const float2*>(p) + i); }

// Bilinear sample of a 1-channel image.
__device__ __forceinline__ float sample1(const float* img, int w, int h, float s, float t) {
  Bilin B = bilin(s, t, w, h);
  return blend1(B, __ldg(img + B.o00), __ldg(img + B.o10), __ldg(img + B.o01), __ldg(img + B.o11));
}
// Bilinear sample of a 4-channel image.
__device__ __forceinline__ float4 sample4(const float* img, int w, int h, float s, float t) {
  Bilin B = bilin(s, t, w, h);
  return blend4(B, ld4(img, B.o00), ld4(img, B.o10), ld4(img, B.o01), ld4(img, B.o11));
}

}  // namespace dev
}  // namespace gi
